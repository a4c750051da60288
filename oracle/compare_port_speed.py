#!/usr/bin/env python3
"""How fast is the oracle port of bssnrhs against the reference's own code?

Test infrastructure, run where the reference tree exists (the GPU host does
not have it, so the benchmark's CPU legs time the port; this script gives the
factor between the two on the same host).  It builds the reference's BSSN
right-hand side twice (oracle/Makefile.ref `timing`): with the reference's
release flags (-O3) and with the port's timing flags (-O3, the host's
instruction set, no floating-point contraction), and times both against the
port (oracle/_build/liboracle_bench.so) on the same stratified sample of the
uneven 20,000-block batch, the same OpenMP loop over blocks and the same
thread count.  The reference keeps its 210 scratch allocations per block.

  python oracle/compare_port_speed.py [--threads N] [--fraction F] [--reps R]
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "tests"))
import oracle_py  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--fraction", type=float, default=1.0 / 100)
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile")], check=True)
    subprocess.run(["make", "-s", "-j8", "-f", os.path.join(HERE, "Makefile.ref"),
                    "REF=" + oracle_py.REF_ROOT, "timing"], check=True)
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "dgb", os.path.join(ROOT, "dendro-5.01_gb300", "dgb.py"))
    dgb = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(dgb)  # pure-Python parts only (block structures, parameters)
    from workloads import repack

    port = oracle_py.Oracle(oracle_py.ORACLE_BENCH_SO)
    blocks = port.synth_blocks(2, 20261203 + 2, dgb.BlockDesc)
    by = {}
    for i, b in enumerate(blocks):
        by.setdefault(b.sz[0], []).append(i)
    k = max(1, int(round(1.0 / a.fraction)))
    idx = sorted(i for lst in by.values() for i in lst[::k])
    sub = repack(dgb, blocks, idx)
    n = dgb.unzipped_size(sub)
    u = [np.zeros(n) for _ in range(24)]
    port.synth_fill(sub, u, 20261203 + 2, 1e-6)
    prm = dgb.params_vector(dgb.default_params(0.1))
    pts = sum((b.sz[0] - 6) * (b.sz[1] - 6) * (b.sz[2] - 6) for b in sub)

    nb = len(sub)
    off = (C.c_ulong * nb)(*[b.offset for b in sub])
    sz = (C.c_uint * (3 * nb))(*[s for b in sub for s in b.sz])
    bf = (C.c_uint * nb)(*[b.bflag for b in sub])
    pmin = np.array([x for b in sub for x in b.ptmin])
    pmax = np.array([x for b in sub for x in b.ptmax])

    def ref_runner(path):
        L = C.CDLL(path)
        L.ref_bssnrhs_blocks.restype = C.c_int
        L.ref_bssnrhs_blocks.argtypes = [C.c_void_p] * 9 + [C.c_int]

        def run(r):
            rp = (C.c_void_p * 24)(*[x.ctypes.data for x in r])
            up = (C.c_void_p * 24)(*[x.ctypes.data for x in u])
            return L.ref_bssnrhs_blocks(rp, up, nb, off, sz, bf, pmin.ctypes.data,
                                        pmax.ctypes.data, prm.ctypes.data, a.threads)
        return run

    runners = {
        "port (liboracle_bench.so: -O3, host ISA, no contraction)":
            lambda r: port.bssnrhs_blocks(r, u, sub, prm, a.threads),
        "reference, release flags (-O3)":
            ref_runner(os.path.join(HERE, "_ref", "libdendro_ref_release.so")),
        "reference, port's timing flags (-O3, host ISA, no contraction)":
            ref_runner(os.path.join(HERE, "_ref", "libdendro_ref_native.so")),
    }
    out, results = {}, {}
    for name, run in runners.items():
        r = [np.zeros(n) for _ in range(24)]
        assert run(r) == 0  # warm-up
        ts = []
        for _ in range(a.reps):
            t0 = time.perf_counter()
            assert run(r) == 0
            ts.append(time.perf_counter() - t0)
        out[name] = pts * 24 / float(np.median(ts))
        results[name] = r
    base = results[next(iter(runners))]
    mask = np.zeros(n, dtype=bool)
    for b in sub:
        nx, ny, nz = b.sz
        m = np.zeros((nz, ny, nx), dtype=bool)
        m[3:-3, 3:-3, 3:-3] = True
        mask[b.offset:b.offset + nx * ny * nz] = m.ravel()
    err = max(float(np.max(np.abs(x[mask] - y[mask])) / max(np.max(np.abs(y[mask])), 1e-300))
              for rr in list(results.values())[1:] for x, y in zip(base, rr))
    names = list(out)
    print(json.dumps({
        "host": os.uname().machine, "threads": a.threads, "blocks": nb, "interior_points": pts,
        "pts_vars_per_s": out,
        "port_over_reference_release": out[names[0]] / out[names[1]],
        "port_over_reference_same_flags": out[names[0]] / out[names[2]],
        "max_normwise_difference": err}, indent=1))


if __name__ == "__main__":
    main()
