#!/usr/bin/env python3
"""Emit csrc/bssn_algebra.cuh: the per-point BSSN right-hand-side algebra.

The system is the one of the reference's generator, CodeGen/bssn.py:36-96
(a_rhs, b_rhs, gt_rhs, chi_rhs, At_rhs, K_rhs, Gt_rhs, B_rhs with eta
constant), built from the tensor helpers of CodeGen/dendro.py (lie :211,
trace_free :317, DiDj :160, laplacian :259, sqr :305, up_up :188,
Christoffels :368-440, compute_ricci :443-527).

The reference expands the whole system symbolically and runs a common
subexpression pass over it ("reduced ops: 4137",
BSSN_GR/src/bssneqs_eta_const_standard_gauge.cpp:1028).  On GB300 the FP64
pipe is the bound, so this generator instead evaluates the same tensor
expressions stage by stage (inverse metric, Christoffels, raised
Christoffels, Ricci, ...) with symmetric components computed once and the
contractions written as FMA chains; the result is algebraically identical
and needs far fewer FP64 instructions.

Accessors the including kernel supplies on `io`:
  io.u(v)        field v at this point (v in bssn::VAR order)
  io.d(slot)     derivative slot (see SLOT_* below)
  io.out(v, x)   right-hand side of field v before KO dissipation
and a `prm` object with l1..l4, lf0, lf1.

With --upwind it emits csrc/bssn_algebra42.cuh instead: the same system for
the BSSN_GR solver's 4th-order binding, where the advective derivative of
every field is the upwinded one (BSSN_GR/include/rhs.h:23-37).  The system
uses advective derivatives only as beta^j ad(j, f) (dendro.py lie :225-248,
vec_j_ad_j :348-353; bssn.py Gt_rhs :86 and B_rhs :100-104), so the kernel
supplies that sum per field, io.d(ADV0 + v), and the algebra reads it in
place of beta^j d_j f.

Run:  python gen_bssn_algebra.py > ../csrc/bssn_algebra.cuh
      python gen_bssn_algebra.py --upwind > ../csrc/bssn_algebra42.cuh
"""
import sys

VARS = ["alpha", "chi", "K", "Gt0", "Gt1", "Gt2", "beta0", "beta1", "beta2",
        "B0", "B1", "B2", "gt0", "gt1", "gt2", "gt3", "gt4", "gt5",
        "At0", "At1", "At2", "At3", "At4", "At5"]
V = {n: i for i, n in enumerate(VARS)}
SYM = [[0, 1, 2], [1, 3, 4], [2, 4, 5]]
PAIRS = [(0, 0), (0, 1), (0, 2), (1, 1), (1, 2), (2, 2)]
# fields with second derivatives (BSSN_GR/scripts/bssnrhs_derivs.h), in VAR order
D2_FIELDS = ["alpha", "chi", "beta0", "beta1", "beta2", "gt0", "gt1", "gt2", "gt3", "gt4", "gt5"]
D2_INDEX = {n: q for q, n in enumerate(D2_FIELDS)}
NUM_GRAD = 72
NUM_D2 = 6 * len(D2_FIELDS)       # xx, xy, xz, yy, yz, zz per field
NUM_DERIV = NUM_GRAD + NUM_D2      # 138
NUM_SLOTS = NUM_DERIV + 24         # + KO sums
ADV0 = NUM_SLOTS                   # upwind form: advection sums beta^j ad_j f per field
NUM_SLOTS_UPWIND = ADV0 + 24


def slot_grad(var, d):
    return 3 * V[var] + d


def slot_d2(var, l, m):
    return NUM_GRAD + 6 * D2_INDEX[var] + SYM[l][m]


class Emitter:
    def __init__(self):
        self.lines = []
        self.loaded = {}

    def let(self, name, expr):
        self.lines.append(f"    const double {name} = {expr};")
        return name

    def d(self, slot):
        """Derivative value, loaded once at first use."""
        if slot not in self.loaded:
            nm = f"d{slot}"
            self.lines.append(f"    const double {nm} = io.d({slot});")
            self.loaded[slot] = nm
        return self.loaded[slot]

    def comment(self, text):
        self.lines.append(f"    // {text}")


def sum_terms(terms):
    """Left-to-right sum of string terms; terms may start with '-'."""
    terms = [t for t in terms if t is not None]
    if not terms:
        return "0.0"
    out = terms[0] if not terms[0].startswith("+") else terms[0][1:]
    for t in terms[1:]:
        if t.startswith("-"):
            out += " - " + t[1:]
        else:
            out += " + " + t
    return out


def generate(upwind=False):
    e = Emitter()

    def adv_of(var, centred):
        """beta^j ad(j, var): the kernel's upwinded sum, or the centred terms
        (centred is called only then, so no unused derivative is loaded)."""
        if upwind:
            return [e.d(ADV0 + V[var])]
        return centred()
    f = {n: f"u_{n}" for n in VARS}
    for n in VARS:
        e.let(f[n], f"io.u({V[n]})")
    a, chi, K = f["alpha"], f["chi"], f["K"]
    Gt = [f["Gt0"], f["Gt1"], f["Gt2"]]
    b = [f["beta0"], f["beta1"], f["beta2"]]
    B = [f["B0"], f["B1"], f["B2"]]
    gsym = [f[f"gt{q}"] for q in range(6)]
    Asym = [f[f"At{q}"] for q in range(6)]
    g = [[gsym[SYM[i][j]] for j in range(3)] for i in range(3)]
    A = [[Asym[SYM[i][j]] for j in range(3)] for i in range(3)]
    gtname = [f"gt{q}" for q in range(6)]
    Atname = [f"At{q}" for q in range(6)]

    def dg(i, j, d):  # d_d gt_ij
        return e.d(slot_grad(gtname[SYM[i][j]], d))

    def dA(i, j, d):
        return e.d(slot_grad(Atname[SYM[i][j]], d))

    def dvec(name, c, d):  # d_d name_c
        return e.d(slot_grad(f"{name}{c}", d))

    def dsc(name, d):
        return e.d(slot_grad(name, d))

    def dd(var, l, m):
        return e.d(slot_d2(var, l, m))

    e.comment("inverse conformal metric: adjugate / determinant (dendro.py:351)")
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
    # off-diagonals doubled, for contractions with symmetric tensors
    for (i, j) in PAIRS:
        if i != j:
            e.let(f"ig2_{i}{j}", f"2.0 * ig{i}{j}")

    def symcontract(X):
        """sum_{ij} ig^ij X_ij for symmetric X given as X[i][j] strings."""
        terms = []
        for (i, j) in PAIRS:
            w = f"ig{i}{j}" if i == j else f"ig2_{i}{j}"
            terms.append(f"{w} * {X[i][j]}")
        return sum_terms(terms)

    e.let("ichi", f"1.0 / {chi}")
    e.let("half_ichi", "0.5 * ichi")
    dchi = [dsc("chi", d) for d in range(3)]
    da = [dsc("alpha", d) for d in range(3)]
    dK = [dsc("K", d) for d in range(3)]

    e.comment("first-kind Christoffels C1_kij = (d_j g_ki + d_i g_kj - d_k g_ij) / 2 "
              "(dendro.py:368-387), the coinciding-index forms reduced")
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
    e.comment("second-kind Christoffels C2^k_ij = ig^kl C1_lij (dendro.py:390-410)")
    C2 = [[[None] * 3 for _ in range(3)] for _ in range(3)]
    for k in range(3):
        for (i, j) in PAIRS:
            nm = e.let(f"C2_{k}{i}{j}", sum_terms([f"{ig[k][l]} * {C1[l][i][j]}" for l in range(3)]))
            C2[k][i][j] = C2[k][j][i] = nm
    e.comment("CalGt^i = ig^kl C2^i_kl (dendro.py:466)")
    CalGt = [e.let(f"CalGt{i}", symcontract(C2[i])) for i in range(3)]
    igdchi = [e.let(f"igdchi{i}", sum_terms([f"{ig[i][m]} * {dchi[m]}" for m in range(3)]))
              for i in range(3)]

    e.comment("raised Christoffels for the quadratic Ricci term")
    C2U = [[[None] * 3 for _ in range(3)] for _ in range(3)]  # sum_l ig^lm C2^k_li
    C1U = [[[None] * 3 for _ in range(3)] for _ in range(3)]  # sum_l ig^ml C1_klj
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

    e.comment("conformal-factor pieces of the Ricci tensor (dendro.py:506-524)")
    ddchi = [[dd("chi", l, m) for m in range(3)] for l in range(3)]
    e.let("chi_c", "1.5 * ichi")  # 3/(2 chi)
    Ychi = [[None] * 3 for _ in range(3)]
    for (k, l) in PAIRS:
        Ychi[k][l] = Ychi[l][k] = e.let(f"Ychi{k}{l}", f"{ddchi[k][l]} - chi_c * {dchi[k]} * {dchi[l]}")
    e.let("trchi", symcontract(Ychi))
    e.let("CalGtdchi", sum_terms([f"{CalGt[m]} * {dchi[m]}" for m in range(3)]))
    e.let("rphi_g", "half_ichi * (trchi - CalGtdchi)")
    e.let("q_ichi2", "0.25 * ichi * ichi")

    e.comment("Ricci tensor R_ij = Rt_ij + Rphi_ij (dendro.py:470-527); on the diagonal the")
    e.comment("two halves of each symmetrised term are equal and are evaluated once")
    R = [[None] * 3 for _ in range(3)]
    for (i, j) in PAIRS:
        t1 = symcontract([[dd(gtname[SYM[i][j]], l, m) for m in range(3)] for l in range(3)])
        e.let(f"t1_{i}{j}", t1)
        c2d = sum_terms([f"{C2[k][j][i]} * {dchi[k]}" for k in range(3)])
        e.let(f"Rphi_{i}{j}", f"half_ichi * ({ddchi[i][j]} - ({c2d})) - q_ichi2 * {dchi[i]} * {dchi[j]}"
              f" + {g[i][j]} * rphi_g")
        if i == j:
            # t2 / 2, t3 / 2 and t4 = 2 A + B of the general form below
            e.let(f"h2_{i}{j}", sum_terms([f"{g[k][i]} * {dvec('Gt', k, i)}" for k in range(3)]))
            e.let(f"h3_{i}{j}", sum_terms([f"{CalGt[k]} * {C1[i][i][k]}" for k in range(3)]))
            e.let(f"t4a_{i}{j}", sum_terms([f"{C2U[k][i][m]} * {C1[i][k][m]}"
                                            for k in range(3) for m in range(3)]))
            e.let(f"t4b_{i}{j}", sum_terms([f"{C2[k][i][m]} * {C1U[k][m][i]}"
                                            for k in range(3) for m in range(3)]))
            R[i][j] = e.let(f"R_{i}{j}", f"-0.5 * t1_{i}{j} + h2_{i}{j} + h3_{i}{j} + "
                                         f"(2.0 * t4a_{i}{j} + t4b_{i}{j}) + Rphi_{i}{j}")
            continue
        t2 = sum_terms([f"{g[k][i]} * {dvec('Gt', k, j)}" for k in range(3)]
                       + [f"{g[k][j]} * {dvec('Gt', k, i)}" for k in range(3)])
        e.let(f"t2_{i}{j}", t2)
        t3 = sum_terms([f"{CalGt[k]} * {dg(i, j, k)}" for k in range(3)])  # C1_ijk + C1_jik = d_k g_ij
        e.let(f"t3_{i}{j}", t3)
        t4 = sum_terms([f"{C2U[k][i][m]} * {C1[j][k][m]}" for k in range(3) for m in range(3)]
                       + [f"{C2U[k][j][m]} * {C1[i][k][m]}" for k in range(3) for m in range(3)]
                       + [f"{C2[k][i][m]} * {C1U[k][m][j]}" for k in range(3) for m in range(3)])
        e.let(f"t4_{i}{j}", t4)
        R[i][j] = R[j][i] = e.let(f"R_{i}{j}",
                                  f"-0.5 * t1_{i}{j} + 0.5 * t2_{i}{j} + 0.5 * t3_{i}{j} + t4_{i}{j} + Rphi_{i}{j}")

    e.comment("D_i D_j alpha with the physical-metric Christoffels C3 (dendro.py:160, :413-440)")
    e.let("igdchi_da", sum_terms([f"{igdchi[l]} * {da[l]}" for l in range(3)]))
    DDa = [[None] * 3 for _ in range(3)]
    for (i, j) in PAIRS:
        c2a = sum_terms([f"{C2[l][i][j]} * {da[l]}" for l in range(3)])
        c3a = f"({c2a}) - half_ichi * ({da[i]} * {dchi[j]} + {da[j]} * {dchi[i]} - {g[i][j]} * igdchi_da)"
        DDa[i][j] = DDa[j][i] = e.let(f"DDa_{i}{j}", f"{dd('alpha', i, j)} - ({c3a})")

    e.let("divb", sum_terms([dvec("beta", k, k) for k in range(3)]))
    e.let("w_divb", "(-2.0 / 3.0) * divb")

    e.comment("lapse and shift (bssn.py:65-72)")
    adv_a = sum_terms(adv_of("alpha", lambda: [f"{b[i]} * {da[i]}" for i in range(3)]))
    e.lines.append(f"    io.out(0, prm.l1 * ({adv_a}) - 2.0 * {a} * {K});")
    e.let("bfac", f"0.75 * (prm.lf0 + prm.lf1 * {a})")
    for i in range(3):
        adv = sum_terms(adv_of(f"beta{i}", lambda: [f"{b[j]} * {dvec('beta', i, j)}" for j in range(3)]))
        e.lines.append(f"    io.out({V['beta0'] + i}, bfac * {B[i]} + prm.l2 * ({adv}));")

    e.comment("chi (bssn.py:76)")
    adv = sum_terms(adv_of("chi", lambda: [f"{b[i]} * {dchi[i]}" for i in range(3)]))
    e.lines.append(f"    io.out(1, {adv} + w_divb * {chi} + (2.0 / 3.0) * ({chi} * {a} * {K}));")

    e.comment("gt: Lie derivative of weight -2/3 minus 2 alpha At (bssn.py:74)")
    for (i, j) in PAIRS:
        terms = adv_of(gtname[SYM[i][j]], lambda: [f"{b[k]} * {dg(i, j, k)}" for k in range(3)])
        terms += [f"{g[i][k]} * {dvec('beta', k, j)}" for k in range(3)]
        terms += [f"{g[k][j]} * {dvec('beta', k, i)}" for k in range(3)]
        terms += [f"w_divb * {g[i][j]}", f"-2.0 * {a} * {A[i][j]}"]
        e.lines.append(f"    io.out({V['gt0'] + SYM[i][j]}, {sum_terms(terms)});")

    e.comment("At (bssn.py:78-80): Lie + chi TF(alpha R - DDalpha) + alpha (K At - 2 At_ik At^k_j)")
    X = [[None] * 3 for _ in range(3)]
    for (i, j) in PAIRS:
        X[i][j] = X[j][i] = e.let(f"X_{i}{j}", f"{a} * {R[i][j]} - {DDa[i][j]}")
    e.let("trX3", f"({symcontract(X)}) * (1.0 / 3.0)")
    AUd = [[None] * 3 for _ in range(3)]
    for k in range(3):
        for j in range(3):
            AUd[k][j] = e.let(f"AUd_{k}{j}", sum_terms([f"{ig[k][l]} * {A[l][j]}" for l in range(3)]))
    for (i, j) in PAIRS:
        lie = adv_of(Atname[SYM[i][j]], lambda: [f"{b[k]} * {dA(i, j, k)}" for k in range(3)])
        lie += [f"{A[i][k]} * {dvec('beta', k, j)}" for k in range(3)]
        lie += [f"{A[k][j]} * {dvec('beta', k, i)}" for k in range(3)]
        lie += [f"w_divb * {A[i][j]}"]
        AA = sum_terms([f"{A[i][k]} * {AUd[k][j]}" for k in range(3)])
        body = (f"{sum_terms(lie)} + {chi} * ({X[i][j]} - {g[i][j]} * trX3)"
                f" + {a} * ({K} * {A[i][j]} - 2.0 * ({AA}))")
        e.lines.append(f"    io.out({V['At0'] + SYM[i][j]}, {body});")

    e.comment("K (bssn.py:82): advection - Laplacian(alpha) + alpha (K^2/3 + At_ij At^ij)")
    AUU = [[None] * 3 for _ in range(3)]
    for (i, j) in PAIRS:
        AUU[i][j] = AUU[j][i] = e.let(f"AUU_{i}{j}",
                                      sum_terms([f"{ig[j][l]} * {AUd[i][l]}" for l in range(3)]))
    # sqr(At) = sum_ij At_ij At^ij (dendro.py:305)
    e.let("sqrA", symcontract_plain(A, AUU))
    e.let("lapa", f"{chi} * ({symcontract(DDa)})")
    advK = sum_terms(adv_of("K", lambda: [f"{b[i]} * {dK[i]}" for i in range(3)]))
    e.lines.append(f"    io.out(2, {advK} - lapa + {a} * ({K} * {K} * (1.0 / 3.0) + sqrA));")

    e.comment("Gt and B (bssn.py:86-104)")
    e.let("a2", f"2.0 * {a}")
    e.let("a3ichi", f"3.0 * {a} * ichi")
    e.let("a43", f"(4.0 / 3.0) * {a}")
    e.let("CalGt_divb", "(2.0 / 3.0) * divb")
    ddb_div = []
    for j in range(3):
        ddb_div.append(e.let(f"ddbdiv{j}", sum_terms([dd(f"beta{k}", j, k) for k in range(3)])))
    for i in range(3):
        terms = adv_of(f"Gt{i}", lambda: [f"{b[j]} * {dvec('Gt', i, j)}" for j in range(3)])
        terms += [f"-{CalGt[j]} * {dvec('beta', i, j)}" for j in range(3)]
        terms += [f"{CalGt[i]} * CalGt_divb"]
        terms += [symcontract([[dd(f"beta{i}", l, m) for m in range(3)] for l in range(3)])]
        terms += [f"(1.0 / 3.0) * ({sum_terms([f'{ig[i][j]} * {ddb_div[j]}' for j in range(3)])})"]
        terms += [f"-2.0 * {AUU[i][j]} * {da[j]}" for j in range(3)]
        terms += [f"a2 * ({symcontract_plain(C2[i], AUU)})"]
        terms += [f"-(a3ichi * {AUU[i][j]} * {dchi[j]} + a43 * {ig[i][j]} * {dK[j]})" for j in range(3)]
        e.let(f"Gtr{i}", sum_terms(terms))
        e.lines.append(f"    io.out({V['Gt0'] + i}, Gtr{i});")
    for i in range(3):
        advB = sum_terms(adv_of(f"B{i}", lambda: [f"{b[j]} * {dvec('B', i, j)}" for j in range(3)]))
        advG = sum_terms(adv_of(f"Gt{i}", lambda: [f"{b[j]} * {dvec('Gt', i, j)}" for j in range(3)]))
        e.lines.append(f"    io.out({V['B0'] + i}, Gtr{i} - eta * {B[i]} + prm.l3 * ({advB})"
                       f" - prm.l4 * ({advG}));")
    return e


def symcontract_plain(X, Y):
    """sum_{jk} X_jk Y_jk for two symmetric tensors given as 3x3 name grids."""
    terms = []
    for (i, j) in PAIRS:
        if i == j:
            terms.append(f"{X[i][j]} * {Y[i][j]}")
        else:
            terms.append(f"2.0 * {X[i][j]} * {Y[i][j]}")
    return sum_terms(terms)


HEADER = """// GENERATED by codegen/gen_bssn_algebra.py -- do not edit by hand.
// Per-point BSSN right-hand side (eta constant, standard gauge) of the
// reference's CodeGen/bssn.py:36-96, evaluated stage by stage.
#pragma once

#define DGB_NUM_GRAD {ng}
#define DGB_NUM_D2 {nd2}
#define DGB_NUM_DERIV {nd}
#define DGB_NUM_SLOTS {ns}
// grad slot of (var v, direction d) = 3 v + d; second derivatives of the
// D2 fields (alpha, chi, beta0..2, gt0..5, in that order q) at
// {ng} + 6 q + (xx, xy, xz, yy, yz, zz); KO sums at {nd} + v.

template <class IO, class PRM>
__device__ __forceinline__ void dgb_bssn_algebra(IO &io, const PRM &prm, const double eta)
{{
"""


HEADER_UPWIND = """// GENERATED by codegen/gen_bssn_algebra.py --upwind -- do not edit by hand.
// Per-point BSSN right-hand side (eta constant, standard gauge) of the
// reference's CodeGen/bssn.py:36-96 for the BSSN_GR solver's 4th-order binding
// (BSSN_GR/include/rhs.h:23-37): the advection terms beta^j ad(j, f) are read
// from slot {adv} + v (the kernel's sums of upwinded derivatives).
#pragma once

#define DGB_B42_ADV0 {adv}
#define DGB_B42_NUM_SLOTS {ns}
// grad slot of (var v, direction d) = 3 v + d; second derivatives of the
// D2 fields (alpha, chi, beta0..2, gt0..5, in that order q) at
// {ng} + 6 q + (xx, xy, xz, yy, yz, zz); KO sums at {nd} + v; advection
// sums at {adv} + v.

template <class IO, class PRM>
__device__ __forceinline__ void dgb_bssn_algebra_upwind(IO &io, const PRM &prm, const double eta)
{{
"""


def main():
    upwind = "--upwind" in sys.argv[1:]
    e = generate(upwind)
    if upwind:
        sys.stdout.write(HEADER_UPWIND.format(ng=NUM_GRAD, nd=NUM_DERIV, adv=ADV0,
                                              ns=NUM_SLOTS_UPWIND))
    else:
        sys.stdout.write(HEADER.format(ng=NUM_GRAD, nd2=NUM_D2, nd=NUM_DERIV, ns=NUM_SLOTS))
    sys.stdout.write("\n".join(e.lines))
    sys.stdout.write("\n}\n")


if __name__ == "__main__":
    main()
