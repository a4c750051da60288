#!/usr/bin/env python3
"""Emit csrc/ccz4_algebra.cuh: the per-point CCZ4 right-hand-side algebra.

The system is the one of the reference's generator,
GR/rhs_scripts/ccz4/ccz4.py:52-117 (a_rhs, b_rhs, gt_rhs, psi_rhs, At_rhs,
K_rhs, Gh_rhs, B_rhs, theta_z4_rhs) with the tensor helpers of
GR/rhs_scripts/ccz4/dendro_ccz4.py (lie :263, DiDj :182, laplacian :309,
trace_free :373, sqr :358, up_up :242, Christoffels :447-536,
compute_ricci :539-589), evaluated stage by stage as for the BSSN system
(gen_bssn_algebra.py).  One deliberate match of the compiled reference: the
Laplacian of alpha in the K equation carries psi^p (CCZ4_GR/src/ccz4eqs.cpp,
1/psi at p = -1), where the generator in the tree writes psi^-p.

Accessors the including kernel supplies on `io`:
  io.u(v)        field v at this point (CCZ4 variable order)
  io.d(slot)     derivative slot (first, advective, second; see the header)
  io.out(v, x)   right-hand side of field v before KO dissipation
and a `prm` object with l1..l4, lf0, lf1, k1, k2, p.

Run:  python gen_ccz4_algebra.py > ../csrc/ccz4_algebra.cuh
"""
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from gen_bssn_algebra import PAIRS, SYM, Emitter, sum_terms, symcontract_plain  # noqa: E402

VARS = ["alpha", "psi", "K", "Gh0", "Gh1", "Gh2", "beta0", "beta1", "beta2",
        "B0", "B1", "B2", "gt0", "gt1", "gt2", "gt3", "gt4", "gt5",
        "At0", "At1", "At2", "At3", "At4", "At5", "theta_z4"]
V = {n: i for i, n in enumerate(VARS)}
NV = len(VARS)
# fields with second derivatives the algebra reads (CCZ4_GR/src/ccz4eqs.cpp)
D2_FIELDS = ["alpha", "psi", "beta0", "beta1", "beta2", "gt0", "gt1", "gt2", "gt3", "gt4", "gt5"]
D2_INDEX = {n: q for q, n in enumerate(D2_FIELDS)}
NUM_GRAD = 3 * NV                  # 75
NUM_ADV = 3 * NV                   # 75
NUM_D2 = 6 * len(D2_FIELDS)        # 66
ADV0 = NUM_GRAD
D20 = NUM_GRAD + NUM_ADV           # 150
NUM_DERIV = D20 + NUM_D2           # 216
NUM_SLOTS = NUM_DERIV + NV         # + KO sums: 241


def slot_grad(var, d):
    return 3 * V[var] + d


def slot_adv(var, d):
    return ADV0 + 3 * V[var] + d


def slot_d2(var, l, m):
    return D20 + 6 * D2_INDEX[var] + SYM[l][m]


def generate():
    e = Emitter()
    f = {n: f"u_{n}" for n in VARS}
    for n in VARS:
        e.let(f[n], f"io.u({V[n]})")
    a, psi, K, th = f["alpha"], f["psi"], f["K"], f["theta_z4"]
    Gh = [f["Gh0"], f["Gh1"], f["Gh2"]]
    b = [f["beta0"], f["beta1"], f["beta2"]]
    B = [f["B0"], f["B1"], f["B2"]]
    g = [[f[f"gt{SYM[i][j]}"] for j in range(3)] for i in range(3)]
    A = [[f[f"At{SYM[i][j]}"] for j in range(3)] for i in range(3)]
    gtname = [f"gt{q}" for q in range(6)]
    Atname = [f"At{q}" for q in range(6)]

    def dg(i, j, d):
        return e.d(slot_grad(gtname[SYM[i][j]], d))

    def dvec(name, c, d):
        return e.d(slot_grad(f"{name}{c}", d))

    def avec(name, c, d):
        return e.d(slot_adv(f"{name}{c}", d))

    def dsc(name, d):
        return e.d(slot_grad(name, d))

    def asc(name, d):
        return e.d(slot_adv(name, d))

    def dd(var, l, m):
        return e.d(slot_d2(var, l, m))

    e.comment("inverse conformal metric: adjugate / determinant (dendro_ccz4.py:426)")
    e.let("m00", f"{g[1][1]} * {g[2][2]} - {g[1][2]} * {g[1][2]}")
    e.let("m01", f"{g[0][2]} * {g[1][2]} - {g[0][1]} * {g[2][2]}")
    e.let("m02", f"{g[0][1]} * {g[1][2]} - {g[0][2]} * {g[1][1]}")
    e.let("m11", f"{g[0][0]} * {g[2][2]} - {g[0][2]} * {g[0][2]}")
    e.let("m12", f"{g[0][1]} * {g[0][2]} - {g[0][0]} * {g[1][2]}")
    e.let("m22", f"{g[0][0]} * {g[1][1]} - {g[0][1]} * {g[0][1]}")
    e.let("det", f"{g[0][0]} * m00 + {g[0][1]} * m01 + {g[0][2]} * m02")
    e.let("idet", "1.0 / det")
    for (i, j) in PAIRS:
        e.let(f"ig{i}{j}", f"m{i}{j} * idet")
    ig = [[f"ig{min(i, j)}{max(i, j)}" for j in range(3)] for i in range(3)]
    for (i, j) in PAIRS:
        if i != j:
            e.let(f"ig2_{i}{j}", f"2.0 * ig{i}{j}")

    def symcontract(X):
        terms = []
        for (i, j) in PAIRS:
            w = f"ig{i}{j}" if i == j else f"ig2_{i}{j}"
            terms.append(f"{w} * {X[i][j]}")
        return sum_terms(terms)

    e.let("ipsi", f"1.0 / {psi}")
    e.let("hp", "0.5 * prm.p * ipsi")
    # psi^-p and psi^p; p = -1 (the reference's P_EXPO) without pow
    e.let("psimp", f"(prm.p == -1.0) ? {psi} : pow({psi}, -prm.p)")
    e.let("psip", f"(prm.p == -1.0) ? ipsi : pow({psi}, prm.p)")
    dpsi = [dsc("psi", d) for d in range(3)]
    da = [dsc("alpha", d) for d in range(3)]
    dK = [dsc("K", d) for d in range(3)]
    dth = [dsc("theta_z4", d) for d in range(3)]

    e.comment("Christoffels of the conformal metric (dendro_ccz4.py:447-500); first kind")
    e.comment("C1_kij = (d_j g_ki + d_i g_kj - d_k g_ij) / 2 with the coinciding-index forms")
    e.comment("reduced")
    C1 = [[[None] * 3 for _ in range(3)] for _ in range(3)]
    for k in range(3):
        for (i, j) in PAIRS:
            if i == j == k:
                expr = f"0.5 * {dg(k, k, k)}"
            elif i == j:  # d_i g_ki - d_k g_ii / 2
                expr = f"{dg(k, i, i)} - 0.5 * {dg(i, i, k)}"
            elif k == i:  # d_j g_kk / 2
                expr = f"0.5 * {dg(k, k, j)}"
            elif k == j:  # d_i g_kk / 2
                expr = f"0.5 * {dg(k, k, i)}"
            else:
                expr = f"0.5 * ({dg(k, i, j)} + {dg(k, j, i)} - {dg(i, j, k)})"
            nm = e.let(f"C1_{k}{i}{j}", expr)
            C1[k][i][j] = C1[k][j][i] = nm
    C2 = [[[None] * 3 for _ in range(3)] for _ in range(3)]
    for k in range(3):
        for (i, j) in PAIRS:
            nm = e.let(f"C2_{k}{i}{j}", sum_terms([f"{ig[k][l]} * {C1[l][i][j]}" for l in range(3)]))
            C2[k][i][j] = C2[k][j][i] = nm
    CalGt = [e.let(f"CalGt{i}", symcontract(C2[i])) for i in range(3)]
    GmC = [e.let(f"GmC{i}", f"{Gh[i]} - {CalGt[i]}") for i in range(3)]
    igdpsi = [e.let(f"igdpsi{i}", sum_terms([f"{ig[i][m]} * {dpsi[m]}" for m in range(3)]))
              for i in range(3)]

    e.comment("raised Christoffels for the quadratic Ricci term")
    C2U = [[[None] * 3 for _ in range(3)] for _ in range(3)]
    C1U = [[[None] * 3 for _ in range(3)] for _ in range(3)]
    for k in range(3):
        for i in range(3):
            for m in range(3):
                C2U[k][i][m] = e.let(f"C2U_{k}{i}{m}",
                                     sum_terms([f"{ig[l][m]} * {C2[k][l][i]}" for l in range(3)]))
    for k in range(3):
        for m in range(3):
            for j in range(3):
                C1U[k][m][j] = e.let(f"C1U_{k}{m}{j}",
                                     sum_terms([f"{ig[m][l]} * {C1[k][l][j]}" for l in range(3)]))

    e.comment("conformal-factor pieces (dendro_ccz4.py:564-585)")
    ddpsi = [[dd("psi", l, m) for m in range(3)] for l in range(3)]
    e.let("cpp2", "0.25 * prm.p * (prm.p + 2.0) * ipsi * ipsi")
    e.let("cpm2", "0.5 * (prm.p - 2.0) * ipsi")
    Yp = [[None] * 3 for _ in range(3)]
    for (k, l) in PAIRS:
        Yp[k][l] = Yp[l][k] = e.let(f"Yp{k}{l}", f"{ddpsi[k][l]} + cpm2 * {dpsi[k]} * {dpsi[l]}")
    e.let("Rtemp", f"hp * (({symcontract(Yp)}) - ({sum_terms([f'{Gh[m]} * {dpsi[m]}' for m in range(3)])}))")
    gG = [e.let(f"gG{i}", sum_terms([f"{GmC[k]} * {g[k][i]}" for k in range(3)])) for i in range(3)]

    e.comment("R_DZ for the trace-free operator: Rt + R_DZ_psi_TF (dendro_ccz4.py:548-589);")
    e.comment("on the diagonal the two halves of each symmetrised term are evaluated once")
    RTF = [[None] * 3 for _ in range(3)]
    for (i, j) in PAIRS:
        t1 = symcontract([[dd(gtname[SYM[i][j]], l, m) for m in range(3)] for l in range(3)])
        e.let(f"t1_{i}{j}", t1)
        c2p = sum_terms([f"{C2[k][i][j]} * {dpsi[k]}" for k in range(3)])
        e.let(f"RpsiTF_{i}{j}", f"-hp * ({ddpsi[i][j]} - ({c2p})) + cpp2 * {dpsi[i]} * {dpsi[j]}"
              f" - hp * ({gG[i]} * {dpsi[j]} + {gG[j]} * {dpsi[i]})")
        if i == j:
            # t2 / 2, t3 / 2 and t4 = 2 A + B of the general form below
            e.let(f"h2_{i}{j}", sum_terms([f"{g[k][i]} * {dvec('Gh', k, i)}" for k in range(3)]))
            e.let(f"h3_{i}{j}", sum_terms([f"{Gh[k]} * {C1[i][i][k]}" for k in range(3)]))
            e.let(f"t4a_{i}{j}", sum_terms([f"{C2U[k][i][m]} * {C1[i][k][m]}"
                                            for k in range(3) for m in range(3)]))
            e.let(f"t4b_{i}{j}", sum_terms([f"{C2[k][i][m]} * {C1U[k][m][i]}"
                                            for k in range(3) for m in range(3)]))
            RTF[i][j] = e.let(f"RTF_{i}{j}", f"-0.5 * t1_{i}{j} + h2_{i}{j} + h3_{i}{j} + "
                                             f"(2.0 * t4a_{i}{j} + t4b_{i}{j}) + RpsiTF_{i}{j}")
            continue
        t2 = sum_terms([f"{g[k][i]} * {dvec('Gh', k, j)}" for k in range(3)]
                       + [f"{g[k][j]} * {dvec('Gh', k, i)}" for k in range(3)])
        e.let(f"t2_{i}{j}", t2)
        t3 = sum_terms([f"{Gh[k]} * {dg(i, j, k)}" for k in range(3)])  # C1_ijk + C1_jik = d_k g_ij
        e.let(f"t3_{i}{j}", t3)
        t4 = sum_terms([f"{C2U[k][i][m]} * {C1[j][k][m]}" for k in range(3) for m in range(3)]
                       + [f"{C2U[k][j][m]} * {C1[i][k][m]}" for k in range(3) for m in range(3)]
                       + [f"{C2[k][i][m]} * {C1U[k][m][j]}" for k in range(3) for m in range(3)])
        e.let(f"t4_{i}{j}", t4)
        RTF[i][j] = RTF[j][i] = e.let(
            f"RTF_{i}{j}", f"-0.5 * t1_{i}{j} + 0.5 * t2_{i}{j} + 0.5 * t3_{i}{j} + t4_{i}{j}"
                           f" + RpsiTF_{i}{j}")
    # trace of R_DZ = R_DZ_TF - gt Rtemp with the inverse metric; tr(ig gt) = 3
    e.let("trRDZ", f"({symcontract(RTF)}) - 3.0 * Rtemp")

    e.comment("D_i D_j alpha with the physical-metric Christoffels C3 (dendro_ccz4.py:182, :503-536)")
    e.let("igdpsi_da", sum_terms([f"{igdpsi[l]} * {da[l]}" for l in range(3)]))
    DDa = [[None] * 3 for _ in range(3)]
    for (i, j) in PAIRS:
        c2a = sum_terms([f"{C2[l][i][j]} * {da[l]}" for l in range(3)])
        c3a = f"({c2a}) + hp * ({da[i]} * {dpsi[j]} + {da[j]} * {dpsi[i]} - {g[i][j]} * igdpsi_da)"
        DDa[i][j] = DDa[j][i] = e.let(f"DDa_{i}{j}", f"{dd('alpha', i, j)} - ({c3a})")

    e.let("divb", sum_terms([dvec("beta", k, k) for k in range(3)]))
    e.let("w_divb", "(-2.0 / 3.0) * divb")
    e.let("Km2th", f"{K} - 2.0 * {th}")

    e.comment("lapse and shift (ccz4.py:59-64)")
    adv_a = sum_terms([f"{b[i]} * {asc('alpha', i)}" for i in range(3)])
    e.lines.append(f"    io.out({V['alpha']}, prm.l1 * ({adv_a}) - 2.0 * {a} * Km2th);")
    e.let("bfac", f"0.75 * (prm.lf0 + prm.lf1 * {a})")
    for i in range(3):
        adv = sum_terms([f"{b[j]} * {avec('beta', i, j)}" for j in range(3)])
        e.lines.append(f"    io.out({V['beta0'] + i}, bfac * {B[i]} + prm.l2 * ({adv}));")

    e.comment("gt: Lie derivative of weight -2/3 minus 2 alpha At (ccz4.py:67)")
    for (i, j) in PAIRS:
        terms = [f"{b[k]} * {e.d(slot_adv(gtname[SYM[i][j]], k))}" for k in range(3)]
        terms += [f"{g[i][k]} * {dvec('beta', k, j)}" for k in range(3)]
        terms += [f"{g[k][j]} * {dvec('beta', k, i)}" for k in range(3)]
        terms += [f"w_divb * {g[i][j]}", f"-2.0 * {a} * {A[i][j]}"]
        e.lines.append(f"    io.out({V['gt0'] + SYM[i][j]}, {sum_terms(terms)});")

    e.comment("psi (ccz4.py:70)")
    adv = sum_terms([f"{b[i]} * {asc('psi', i)}" for i in range(3)])
    e.lines.append(f"    io.out({V['psi']}, {adv} + (2.0 / 3.0) * {psi} * (divb - {a} * {K}) / prm.p);")

    e.comment("At (ccz4.py:77): Lie + psi^-p TF(alpha R_DZ - DDalpha) + alpha ((K - 2 theta) At - 2 At_ik At^k_j)")
    X = [[None] * 3 for _ in range(3)]
    for (i, j) in PAIRS:
        X[i][j] = X[j][i] = e.let(f"X_{i}{j}", f"{a} * {RTF[i][j]} - {DDa[i][j]}")
    e.let("trX3", f"({symcontract(X)}) * (1.0 / 3.0)")
    AUd = [[None] * 3 for _ in range(3)]
    for k in range(3):
        for j in range(3):
            AUd[k][j] = e.let(f"AUd_{k}{j}", sum_terms([f"{ig[k][l]} * {A[l][j]}" for l in range(3)]))
    for (i, j) in PAIRS:
        lie = [f"{b[k]} * {e.d(slot_adv(Atname[SYM[i][j]], k))}" for k in range(3)]
        lie += [f"{A[i][k]} * {dvec('beta', k, j)}" for k in range(3)]
        lie += [f"{A[k][j]} * {dvec('beta', k, i)}" for k in range(3)]
        lie += [f"w_divb * {A[i][j]}"]
        AA = sum_terms([f"{A[i][k]} * {AUd[k][j]}" for k in range(3)])
        body = (f"{sum_terms(lie)} + psimp * ({X[i][j]} - {g[i][j]} * trX3)"
                f" + {a} * (Km2th * {A[i][j]} - 2.0 * ({AA}))")
        e.lines.append(f"    io.out({V['At0'] + SYM[i][j]}, {body});")

    e.comment("K (ccz4.py:81); the Laplacian of alpha with psi^p as the compiled reference")
    AUU = [[None] * 3 for _ in range(3)]
    for (i, j) in PAIRS:
        AUU[i][j] = AUU[j][i] = e.let(f"AUU_{i}{j}",
                                      sum_terms([f"{ig[j][l]} * {AUd[i][l]}" for l in range(3)]))
    e.let("sqrA", symcontract_plain(A, AUU))
    e.let("lapa", f"psip * ({symcontract(DDa)})")
    advK = sum_terms([f"{b[i]} * {asc('K', i)}" for i in range(3)])
    e.lines.append(f"    io.out({V['K']}, {advK} - lapa + {a} * (psimp * trRDZ + {K} * Km2th"
                   f" - 3.0 * prm.k1 * (1.0 + prm.k2) * {th}));")

    e.comment("Gh and B (ccz4.py:88-102)")
    e.let("a2", f"2.0 * {a}")
    e.let("a3p_ipsi", f"3.0 * {a} * prm.p * ipsi")
    e.let("a43", f"(4.0 / 3.0) * {a}")
    e.let("Gh_divb", "(2.0 / 3.0) * divb")
    e.let("kfac", f"{a} * (prm.k1 + (2.0 / 3.0) * {K})")
    ddb_div = []
    for j in range(3):
        ddb_div.append(e.let(f"ddbdiv{j}", sum_terms([dd(f"beta{k}", j, k) for k in range(3)])))
    for i in range(3):
        terms = [f"{b[j]} * {avec('Gh', i, j)}" for j in range(3)]
        terms += [f"-{Gh[j]} * {dvec('beta', i, j)}" for j in range(3)]
        terms += [f"{Gh[i]} * Gh_divb"]
        terms += [symcontract([[dd(f"beta{i}", l, m) for m in range(3)] for l in range(3)])]
        terms += [f"(1.0 / 3.0) * ({sum_terms([f'{ig[i][j]} * {ddb_div[j]}' for j in range(3)])})"]
        terms += [f"-2.0 * {AUU[i][j]} * {da[j]}" for j in range(3)]
        terms += [f"a2 * ({symcontract_plain(C2[i], AUU)})"]
        terms += [f"a3p_ipsi * {AUU[i][j]} * {dpsi[j]}" for j in range(3)]
        terms += [f"-a43 * {ig[i][j]} * {dK[j]}" for j in range(3)]
        terms += [f"2.0 * {ig[i][j]} * ({a} * {dth[j]} - {th} * {da[j]})" for j in range(3)]
        terms += [f"-kfac * {GmC[i]}"]
        e.let(f"Ghr{i}", sum_terms(terms))
        e.lines.append(f"    io.out({V['Gh0'] + i}, Ghr{i});")
    for i in range(3):
        advB = sum_terms([f"{b[j]} * {avec('B', i, j)}" for j in range(3)])
        advG = sum_terms([f"{b[j]} * {avec('Gh', i, j)}" for j in range(3)])
        e.lines.append(f"    io.out({V['B0'] + i}, Ghr{i} - eta * {B[i]} + prm.l3 * ({advB})"
                       f" - prm.l4 * ({advG}));")

    e.comment("theta_z4 (ccz4.py:104)")
    advT = sum_terms([f"{b[i]} * {asc('theta_z4', i)}" for i in range(3)])
    GdA = sum_terms([f"{GmC[i]} * {da[i]}" for i in range(3)])
    e.lines.append(f"    io.out({V['theta_z4']}, {advT} + 0.5 * {a} * (psimp * trRDZ"
                   f" + (2.0 / 3.0) * {K} * {K} - sqrA - 2.0 * {th} * {K})"
                   f" - 0.5 * psimp * ({GdA}) - {a} * (prm.k1 * (2.0 + prm.k2) * {th}));")
    return e


HEADER = """// GENERATED by codegen/gen_ccz4_algebra.py -- do not edit by hand.
// Per-point CCZ4 right-hand side of the reference's
// GR/rhs_scripts/ccz4/ccz4.py:52-117, evaluated stage by stage.
#pragma once

#define DGB_CCZ4_NUM_GRAD {ng}
#define DGB_CCZ4_ADV0 {a0}
#define DGB_CCZ4_D20 {d20}
#define DGB_CCZ4_NUM_DERIV {nd}
#define DGB_CCZ4_NUM_SLOTS {ns}
// grad slot of (var v, direction d) = 3 v + d; advective (upwind) slot =
// {a0} + 3 v + d; second derivatives of the D2 fields (alpha, psi,
// beta0..2, gt0..5, in that order q) at {d20} + 6 q + (xx, xy, xz, yy, yz, zz);
// KO sums at {nd} + v.

template <class IO, class PRM>
__device__ __forceinline__ void dgb_ccz4_algebra(IO &io, const PRM &prm, const double eta)
{{
"""


def main():
    e = generate()
    sys.stdout.write(HEADER.format(ng=NUM_GRAD, a0=ADV0, d20=D20, nd=NUM_DERIV, ns=NUM_SLOTS))
    sys.stdout.write("\n".join(e.lines))
    sys.stdout.write("\n}\n")


if __name__ == "__main__":
    main()
