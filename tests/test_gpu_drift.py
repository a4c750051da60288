"""Mixed precision (FP32 stencils and KO) against FP64 over an evolution on
an octree: per-field state error after 20 RK4 steps and the drift of the
Hamiltonian / momentum constraint L2 norms the solver reports
(BSSN_GR/src/bssnCtx.cpp:332-365), mixed within 2x of FP64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STEPS = 20


def test_mixed_precision_drift_small_octree(dgb, gpu):
    torch = gpu
    m = dgb.Mesh(dgb.mesh_params(max_level=7, min_level=4, fine_radius=1.0))
    plan = dgb.Plan(m.blocks, dgb.default_params(0.4))
    uz = dgb.UnzipPlan(m.operator(), m.ndof)
    host = [np.empty(m.ndof) for _ in range(24)]
    dgb.synth_fill_points(m.dof_coords(), host, 20261206, 1e-6)
    U = [torch.zeros(m.nunzipped, dtype=torch.float64, device="cuda") for _ in range(24)]
    Cu = [torch.zeros(m.nunzipped, dtype=torch.float64, device="cuda") for _ in range(6)]
    Cz = [torch.zeros(m.ndof, dtype=torch.float64, device="cuda") for _ in range(6)]
    bufs = ([t.data_ptr() for t in U], [t.data_ptr() for t in Cu], [t.data_ptr() for t in Cz])
    dt = 0.25 * 64.0 / (2 ** 7 * 6)
    l2, final = {}, {}
    for prec in (dgb.PREC_FP64, dgb.PREC_MIXED):
        st = dgb.Stepper(plan, uz, prec)
        ds = [torch.from_numpy(a).cuda() for a in host]
        ptrs = [t.data_ptr() for t in ds]
        first = dgb.constraint_report(plan, uz, ptrs, *bufs, m.ndof)
        st.step(ptrs, dt, nsteps=STEPS)
        last = dgb.constraint_report(plan, uz, ptrs, *bufs, m.ndof)
        l2[prec], final[prec] = (np.array(first), np.array(last)), ds
        st.close()
    f0, f1 = l2[dgb.PREC_FP64]
    m0, m1 = l2[dgb.PREC_MIXED]
    assert np.array_equal(f0, m0)  # same initial state, same report
    assert np.all(np.isfinite(f1)) and np.all(np.isfinite(m1))
    assert np.all(f1 != f0)  # the constraints do evolve
    ratio = np.abs(m1 - m0) / np.abs(f1 - f0)
    assert np.all(ratio <= 2.0) and np.all(ratio >= 0.5), ratio
    for v in range(24):
        a, b = final[dgb.PREC_MIXED][v], final[dgb.PREC_FP64][v]
        err = float((a - b).abs().max()) / float(b.abs().max())
        assert err <= 1e-7, (dgb.VAR_NAMES[v], err)
    uz.close()
    plan.close()
    m.close()
