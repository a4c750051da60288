// Host-side octree mesh for the full-step path: a 2:1-balanced octree
// refined around the punctures, its regular blocks, the continuous-Galerkin
// node numbering (the "zipped" vector) and the unzip / zip operators.
//
// What it restates (the reference's own mesh needs MPI and LAPACK and is not
// compiled here; see the oracle notes):
//   octree + 2:1 balance        ot::Mesh construction (src/mesh.cpp:283),
//                               balance across faces, edges and corners
//   blocks                      octree2BlockDecomposition (src/octUtils.cpp:556)
//                               / performBlocksSetup (src/mesh.cpp:8640-8790):
//                               maximal aligned cubes of 2^k x 2^k x 2^k leaves of
//                               one level (k <= 3), side p*2^k + 1 + 6 (src/block.cpp:50),
//                               offsets = exclusive prefix sum (src/mesh.cpp:8667-8672),
//                               bflag = domain faces touched (src/mesh.cpp:8701-8738)
//   zipped vector               one value per independent element node: a node
//                               position is independent when it lies on the node
//                               lattice of every leaf whose closure contains it;
//                               the others are hanging
//   Mesh::unzip                 every padded point inside the domain gets the mesh
//   (include/mesh.tcc:7436-8690) field at its position: the degree-p Lagrange
//                               interpolant of the coarsest leaf containing it,
//                               whose hanging nodes are themselves interpolated
//                               from coarser leaves.  This equals the reference's
//                               element copy, same-level padding copy, coarser
//                               neighbour parent->child interpolation
//                               (FEM/include/refel.h:249-296), finer neighbour
//                               child->parent injection (mesh.tcc:7399-7433) and
//                               edge/corner padding, written as one rule.
//   Mesh::zip                   every independent node takes the block value
//   (include/mesh.tcc:3775-3822) at its position from one owning block (the
//                               finest block holding it in its interior, first
//                               in block order on ties).
// Points outside the domain are not written by unzip (they are the padding
// beyond domain faces of boundary blocks).
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/dendro_gb300.h"

namespace {

constexpr int P = 6;  // element order

struct Leaf {
    uint32_t a[3];  // anchor in node-lattice units
    int lev;
};

inline uint64_t key(int lev, uint32_t x, uint32_t y, uint32_t z)
{
    return ((uint64_t)lev << 48) | ((uint64_t)x << 32) | ((uint64_t)y << 16) | (uint64_t)z;
}
inline uint64_t pkey(uint32_t x, uint32_t y, uint32_t z)
{
    return ((uint64_t)x << 32) | ((uint64_t)y << 16) | (uint64_t)z;
}

struct Term {
    uint32_t dof;
    double w;
};

}  // namespace

struct dgb_mesh {
    dgb_mesh_params prm;
    int D = 0;          // max level
    uint32_t N = 0;     // node-lattice units across the domain = P * 2^D
    double unit = 0.0;  // domain length per lattice unit
    std::vector<Leaf> leaves;
    std::unordered_map<uint64_t, uint32_t> leaf_of;  // key(lev, anchor) -> leaf index
    std::vector<dgb_block_desc> blocks;
    std::vector<int> block_lev;
    std::vector<uint32_t> block_anchor;  // 3 per block (lattice units)
    std::unordered_map<uint64_t, uint32_t> dof_of;  // pkey(position) -> dof
    std::vector<uint32_t> dof_pos;                   // 3 per dof
    std::vector<uint64_t> unzipped_total;
    // unzip operator
    std::vector<uint32_t> copy_src;     // per padded point: dof, or sentinel
    std::vector<uint64_t> interp_dst;   // padded point of each interpolation row
    std::vector<uint64_t> interp_ptr;   // CSR
    std::vector<uint32_t> interp_col;
    std::vector<double> interp_w;
    std::vector<uint64_t> zip_src;      // per dof: padded point it is read from
    std::unordered_map<uint64_t, std::vector<Term>> memo;  // hanging-node rows

    uint32_t S(int lev) const { return (uint32_t)P << (D - lev); }   // leaf size
    uint32_t sp(int lev) const { return 1u << (D - lev); }          // node spacing

    // Leaf containing the point q + eps * dir (dir components in {-1, +1}),
    // or -1 outside the domain.
    // hint: a level to try first (2:1 balance keeps neighbours within one level)
    int64_t leaf_at(const int64_t q[3], const int dir[3], int hint = -1) const
    {
        int64_t c[3];
        for (int a = 0; a < 3; a++) {
            c[a] = dir[a] < 0 ? q[a] - 1 : q[a];
            if (c[a] < 0 || c[a] >= (int64_t)N) return -1;
        }
        auto probe = [&](int lev) -> int64_t {
            const uint32_t s = S(lev);
            auto it = leaf_of.find(key(lev, (uint32_t)(c[0] / s * s), (uint32_t)(c[1] / s * s),
                                       (uint32_t)(c[2] / s * s)));
            return it != leaf_of.end() ? (int64_t)it->second : -1;
        };
        if (hint >= 0) {
            for (int lev : {hint, hint - 1, hint + 1}) {
                if (lev < 0 || lev > D) continue;
                const int64_t e = probe(lev);
                if (e >= 0) return e;
            }
        }
        for (int lev = D; lev >= 0; lev--) {
            const int64_t e = probe(lev);
            if (e >= 0) return e;
        }
        return -1;
    }
    // Leaf whose half-open box holds the lattice point c (inside the domain).
    int64_t leaf_holding(const int64_t c[3]) const
    {
        const int dir[3] = {1, 1, 1};
        return leaf_at(c, dir);
    }
    bool on_lattice(const Leaf &e, const int64_t q[3]) const
    {
        const int64_t s = sp(e.lev);
        for (int a = 0; a < 3; a++)
            if ((q[a] - (int64_t)e.a[a]) % s != 0) return false;
        return true;
    }
    // Coarsest leaf whose closure holds q; also whether q is an independent node.
    int64_t coarsest_at(const int64_t q[3], bool *independent, int hint = -1) const
    {
        int64_t best = -1;
        bool indep = true;
        for (int c = 0; c < 8; c++) {
            const int dir[3] = {(c & 1) ? 1 : -1, (c & 2) ? 1 : -1, (c & 4) ? 1 : -1};
            const int64_t e = leaf_at(q, dir, hint);
            if (e >= 0) hint = leaves[e].lev;
            if (e < 0) continue;
            if (!on_lattice(leaves[e], q)) indep = false;
            if (best < 0 || leaves[e].lev < leaves[best].lev) best = e;
        }
        if (independent) *independent = indep;
        return best;
    }
};

namespace {

// Lagrange basis weight of node i (uniform nodes 0..P) at xi.
double lagrange(int i, double xi)
{
    double num = 1.0, den = 1.0;
    for (int m = 0; m <= P; m++) {
        if (m == i) continue;
        num *= (xi - m);
        den *= (double)(i - m);
    }
    return num / den;
}

// Field at lattice point q as a combination of independent node values.
void eval_point(dgb_mesh &M, const int64_t q[3], std::vector<Term> &out, double scale, int hint)
{
    bool indep = false;
    const int64_t e = M.coarsest_at(q, &indep, hint);
    if (e < 0) return;
    if (indep) {
        auto it = M.dof_of.find(pkey((uint32_t)q[0], (uint32_t)q[1], (uint32_t)q[2]));
        if (it != M.dof_of.end()) {
            out.push_back({it->second, scale});
            return;
        }
    }
    const uint64_t mk = pkey((uint32_t)q[0], (uint32_t)q[1], (uint32_t)q[2]);
    auto mit = M.memo.find(mk);
    if (mit == M.memo.end()) {
        const Leaf L = M.leaves[e];
        const int64_t s = M.sp(L.lev);
        int idx[3][P + 1];
        double wt[3][P + 1];
        int cnt[3];
        for (int a = 0; a < 3; a++) {
            const int64_t d = q[a] - (int64_t)L.a[a];
            if (d % s == 0) {
                cnt[a] = 1;
                idx[a][0] = (int)(d / s);
                wt[a][0] = 1.0;
            } else {
                cnt[a] = P + 1;
                const double xi = (double)d / (double)s;
                for (int i = 0; i <= P; i++) {
                    idx[a][i] = i;
                    wt[a][i] = lagrange(i, xi);
                }
            }
        }
        std::vector<Term> row;
        for (int k = 0; k < cnt[2]; k++)
            for (int j = 0; j < cnt[1]; j++)
                for (int i = 0; i < cnt[0]; i++) {
                    const double w = wt[0][i] * wt[1][j] * wt[2][k];
                    const int64_t n[3] = {(int64_t)L.a[0] + s * idx[0][i],
                                          (int64_t)L.a[1] + s * idx[1][j],
                                          (int64_t)L.a[2] + s * idx[2][k]};
                    if (n[0] == q[0] && n[1] == q[1] && n[2] == q[2]) {
                        // q itself is a hanging node of the coarsest leaf: cannot happen,
                        // the coarsest leaf holds q on its lattice only if q is independent
                        continue;
                    }
                    eval_point(M, n, row, w, L.lev);
                }
        // merge duplicates
        std::sort(row.begin(), row.end(), [](const Term &x, const Term &y) { return x.dof < y.dof; });
        std::vector<Term> merged;
        for (const Term &t : row) {
            if (!merged.empty() && merged.back().dof == t.dof)
                merged.back().w += t.w;
            else
                merged.push_back(t);
        }
        mit = M.memo.emplace(mk, std::move(merged)).first;
    }
    for (const Term &t : mit->second) out.push_back({t.dof, t.w * scale});
}

int target_level(const dgb_mesh &M, const Leaf &o)
{
    // distance (domain units) from the leaf box to the nearest puncture
    const dgb_mesh_params &p = M.prm;
    double best = 1e300;
    const double s = M.S(o.lev) * M.unit;
    for (int q = 0; q < p.num_punctures; q++) {
        double d2 = 0.0;
        for (int a = 0; a < 3; a++) {
            const double lo = p.domain_min[a] + o.a[a] * M.unit, hi = lo + s;
            const double c = p.puncture[q][a];
            const double d = c < lo ? lo - c : (c > hi ? c - hi : 0.0);
            d2 += d * d;
        }
        best = std::min(best, sqrt(d2));
    }
    // finest level within fine_radius, one level coarser per doubling of the distance
    int lev = p.max_level;
    double r = p.fine_radius;
    while (best >= r && lev > p.min_level) {
        lev--;
        r *= 2.0;
    }
    return lev;
}

}  // namespace

extern "C" {

dgb_status dgb_mesh_create(const dgb_mesh_params *prm, dgb_mesh **out)
{
    if (!prm || !out) return DGB_ERR_INVALID;
    *out = nullptr;
    if (prm->ele_order != P || prm->max_level < prm->min_level || prm->max_level > 12 ||
        prm->min_level < 1 || prm->num_punctures < 0 || prm->num_punctures > 4 ||
        prm->max_block_refine < 0 || prm->max_block_refine > 3)
        return DGB_ERR_INVALID;
    for (int a = 0; a < 3; a++)
        if (!(prm->domain_max[a] > prm->domain_min[a])) return DGB_ERR_INVALID;
    if (prm->domain_max[0] - prm->domain_min[0] != prm->domain_max[1] - prm->domain_min[1] ||
        prm->domain_max[0] - prm->domain_min[0] != prm->domain_max[2] - prm->domain_min[2])
        return DGB_ERR_INVALID;  // cubic domain: one spacing per level
    dgb_mesh *M = new dgb_mesh();
    M->prm = *prm;
    M->D = prm->max_level;
    M->N = (uint32_t)P << M->D;
    M->unit = (prm->domain_max[0] - prm->domain_min[0]) / (double)M->N;

    // ---- refinement: recursive from the root
    std::vector<Leaf> work{Leaf{{0, 0, 0}, 0}};
    std::vector<Leaf> leaves;
    while (!work.empty()) {
        Leaf o = work.back();
        work.pop_back();
        if (o.lev < target_level(*M, o)) {
            const uint32_t h = M->S(o.lev + 1);
            for (int c = 0; c < 8; c++)
                work.push_back(Leaf{{o.a[0] + ((c & 1) ? h : 0), o.a[1] + ((c & 2) ? h : 0),
                                     o.a[2] + ((c & 4) ? h : 0)}, o.lev + 1});
        } else {
            leaves.push_back(o);
        }
    }
    // ---- 2:1 balance across faces, edges and corners
    auto rebuild_index = [&]() {
        M->leaf_of.clear();
        M->leaf_of.reserve(leaves.size() * 2);
        for (size_t i = 0; i < leaves.size(); i++)
            M->leaf_of[key(leaves[i].lev, leaves[i].a[0], leaves[i].a[1], leaves[i].a[2])] = (uint32_t)i;
        M->leaves = leaves;
    };
    for (;;) {
        rebuild_index();
        std::vector<char> refine(leaves.size(), 0);
        bool any = false;
        for (size_t i = 0; i < leaves.size(); i++) {
            const Leaf &e = leaves[i];
            const int64_t s = M->S(e.lev);
            for (int dz = -1; dz <= 1; dz++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dx = -1; dx <= 1; dx++) {
                        if (!dx && !dy && !dz) continue;
                        const int d[3] = {dx, dy, dz};
                        int64_t c[3];
                        bool inside = true;
                        for (int a = 0; a < 3; a++) {
                            c[a] = (int64_t)e.a[a] + (d[a] < 0 ? -1 : d[a] > 0 ? s : s / 2);
                            if (c[a] < 0 || c[a] >= (int64_t)M->N) inside = false;
                        }
                        if (!inside) continue;
                        const int64_t nb = M->leaf_holding(c);
                        if (nb >= 0 && leaves[nb].lev < e.lev - 1) {
                            refine[nb] = 1;
                            any = true;
                        }
                    }
        }
        if (!any) break;
        std::vector<Leaf> next;
        next.reserve(leaves.size() + 8);
        for (size_t i = 0; i < leaves.size(); i++) {
            if (!refine[i]) {
                next.push_back(leaves[i]);
                continue;
            }
            const Leaf o = leaves[i];
            const uint32_t h = M->S(o.lev + 1);
            for (int c = 0; c < 8; c++)
                next.push_back(Leaf{{o.a[0] + ((c & 1) ? h : 0), o.a[1] + ((c & 2) ? h : 0),
                                     o.a[2] + ((c & 4) ? h : 0)}, o.lev + 1});
        }
        leaves.swap(next);
    }
    // Morton order of the leaves (by anchor bits, coarse-to-fine interleave)
    auto morton = [&](const Leaf &l) {
        uint64_t m = 0;
        for (int b = 15; b >= 0; b--)
            for (int a = 2; a >= 0; a--) m = (m << 1) | ((l.a[a] / P) >> b & 1u);
        return m;
    };
    std::sort(leaves.begin(), leaves.end(), [&](const Leaf &x, const Leaf &y) {
        const uint64_t mx = morton(x), my = morton(y);
        return mx != my ? mx < my : x.lev < y.lev;
    });
    rebuild_index();

    // ---- blocks: maximal aligned cubes of 2^k leaves of one level
    std::vector<char> used(leaves.size(), 0);
    uint64_t off = 0;
    const int kmax = prm->max_block_refine;
    for (size_t i = 0; i < leaves.size(); i++) {
        if (used[i]) continue;
        const Leaf e = leaves[i];
        int kbest = 0;
        uint32_t anc[3] = {e.a[0], e.a[1], e.a[2]};
        for (int k = std::min(kmax, e.lev); k >= 1; k--) {
            const uint32_t sa = M->S(e.lev - k);
            const uint32_t A[3] = {e.a[0] / sa * sa, e.a[1] / sa * sa, e.a[2] / sa * sa};
            if (A[0] != e.a[0] || A[1] != e.a[1] || A[2] != e.a[2]) continue;  // e must be the first leaf
            const uint32_t s = M->S(e.lev), m = 1u << k;
            bool ok = true;
            for (uint32_t z = 0; z < m && ok; z++)
                for (uint32_t y = 0; y < m && ok; y++)
                    for (uint32_t x = 0; x < m && ok; x++) {
                        auto it = M->leaf_of.find(key(e.lev, A[0] + x * s, A[1] + y * s, A[2] + z * s));
                        if (it == M->leaf_of.end() || used[it->second]) ok = false;
                    }
            if (ok) {
                kbest = k;
                anc[0] = A[0]; anc[1] = A[1]; anc[2] = A[2];
                break;
            }
        }
        const uint32_t s = M->S(e.lev), m = 1u << kbest;
        for (uint32_t z = 0; z < m; z++)
            for (uint32_t y = 0; y < m; y++)
                for (uint32_t x = 0; x < m; x++)
                    used[M->leaf_of[key(e.lev, anc[0] + x * s, anc[1] + y * s, anc[2] + z * s)]] = 1;
        dgb_block_desc b;
        memset(&b, 0, sizeof b);
        const uint32_t side = (uint32_t)P * m + 1 + 6;
        const double h = M->sp(e.lev) * M->unit;
        for (int a = 0; a < 3; a++) {
            b.sz[a] = side;
            const double x0 = prm->domain_min[a] + anc[a] * M->unit;
            b.ptmin[a] = x0 - 3 * h;
            b.ptmax[a] = x0 + (double)(P * m) * h + 3 * h;
            if (anc[a] == 0) b.bflag |= 1u << (2 * a);
            if (anc[a] + s * m == M->N) b.bflag |= 1u << (2 * a + 1);
        }
        b.offset = off;
        off += (uint64_t)side * side * side;
        M->blocks.push_back(b);
        M->block_lev.push_back(e.lev);
        M->block_anchor.insert(M->block_anchor.end(), anc, anc + 3);
    }

    // ---- independent nodes (the zipped vector), leaf by leaf
    M->dof_of.reserve(leaves.size() * 250);
    for (size_t i = 0; i < leaves.size(); i++) {
        const Leaf &e = leaves[i];
        const int64_t s = M->sp(e.lev);
        for (int k = 0; k <= P; k++)
            for (int j = 0; j <= P; j++)
                for (int ii = 0; ii <= P; ii++) {
                    const int64_t q[3] = {(int64_t)e.a[0] + s * ii, (int64_t)e.a[1] + s * j,
                                          (int64_t)e.a[2] + s * k};
                    const uint64_t pk = pkey((uint32_t)q[0], (uint32_t)q[1], (uint32_t)q[2]);
                    if (M->dof_of.count(pk)) continue;
                    bool indep = true;
                    if (ii == 0 || ii == P || j == 0 || j == P || k == 0 || k == P)
                        M->coarsest_at(q, &indep, e.lev);  // inner nodes belong to e alone
                    if (!indep) continue;
                    const uint32_t id = (uint32_t)M->dof_pos.size() / 3;
                    M->dof_of.emplace(pk, id);
                    M->dof_pos.push_back((uint32_t)q[0]);
                    M->dof_pos.push_back((uint32_t)q[1]);
                    M->dof_pos.push_back((uint32_t)q[2]);
                }
    }
    const uint64_t ndof = M->dof_pos.size() / 3;

    // ---- unzip operator and zip owners
    const uint32_t SENT = 0xFFFFFFFFu;
    M->copy_src.assign(off, SENT);
    M->zip_src.assign(ndof, ~0ull);
    std::vector<int> owner_lev(ndof, -1);
    M->interp_ptr.push_back(0);
    std::vector<Term> row;
    for (size_t b = 0; b < M->blocks.size(); b++) {
        const dgb_block_desc &B = M->blocks[b];
        const int lev = M->block_lev[b];
        const int64_t s = M->sp(lev);
        const uint32_t *A = &M->block_anchor[3 * b];
        const int n = (int)B.sz[0];
        for (int k = 0; k < n; k++)
            for (int j = 0; j < n; j++)
                for (int i = 0; i < n; i++) {
                    const int64_t q[3] = {(int64_t)A[0] + s * (i - 3), (int64_t)A[1] + s * (j - 3),
                                          (int64_t)A[2] + s * (k - 3)};
                    bool inside = true;
                    for (int a = 0; a < 3; a++)
                        if (q[a] < 0 || q[a] > (int64_t)M->N) inside = false;
                    if (!inside) continue;
                    const uint64_t dst = B.offset + (uint64_t)i + (uint64_t)n * (j + (uint64_t)n * k);
                    row.clear();
                    eval_point(*M, q, row, 1.0, lev);
                    if (row.size() == 1 && row[0].w == 1.0) {
                        M->copy_src[dst] = row[0].dof;
                        const bool interior = i >= 3 && i < n - 3 && j >= 3 && j < n - 3 && k >= 3 && k < n - 3;
                        if (interior && lev > owner_lev[row[0].dof]) {
                            owner_lev[row[0].dof] = lev;
                            M->zip_src[row[0].dof] = dst;
                        }
                    } else if (!row.empty()) {
                        M->interp_dst.push_back(dst);
                        for (const Term &t : row) {
                            M->interp_col.push_back(t.dof);
                            M->interp_w.push_back(t.w);
                        }
                        M->interp_ptr.push_back(M->interp_col.size());
                    }
                }
    }
    for (uint64_t d = 0; d < ndof; d++)
        if (M->zip_src[d] == ~0ull) {
            delete M;
            return DGB_ERR_INVALID;  // an independent node without an owning block
        }
    M->memo.clear();
    *out = M;
    return DGB_OK;
}

dgb_status dgb_mesh_destroy(dgb_mesh *M)
{
    delete M;
    return DGB_OK;
}

dgb_status dgb_mesh_sizes(const dgb_mesh *M, uint64_t *sizes)
{
    if (!M || !sizes) return DGB_ERR_INVALID;
    sizes[0] = M->leaves.size();
    sizes[1] = M->dof_pos.size() / 3;
    sizes[2] = M->blocks.size();
    sizes[3] = M->copy_src.size();
    sizes[4] = M->interp_dst.size();
    sizes[5] = M->interp_col.size();
    return DGB_OK;
}

dgb_status dgb_mesh_blocks(const dgb_mesh *M, dgb_block_desc *out)
{
    if (!M || !out) return DGB_ERR_INVALID;
    memcpy(out, M->blocks.data(), M->blocks.size() * sizeof(dgb_block_desc));
    return DGB_OK;
}

dgb_status dgb_mesh_dof_coords(const dgb_mesh *M, double *xyz)
{
    if (!M || !xyz) return DGB_ERR_INVALID;
    const size_t n = M->dof_pos.size() / 3;
    for (size_t d = 0; d < n; d++)
        for (int a = 0; a < 3; a++)
            xyz[3 * d + a] = M->prm.domain_min[a] + M->dof_pos[3 * d + a] * M->unit;
    return DGB_OK;
}

dgb_status dgb_mesh_leaf_levels(const dgb_mesh *M, uint8_t *lev, uint32_t *anchor)
{
    if (!M) return DGB_ERR_INVALID;
    for (size_t i = 0; i < M->leaves.size(); i++) {
        if (lev) lev[i] = (uint8_t)M->leaves[i].lev;
        if (anchor)
            for (int a = 0; a < 3; a++) anchor[3 * i + a] = M->leaves[i].a[a];
    }
    return DGB_OK;
}

dgb_status dgb_mesh_unzip_operator(const dgb_mesh *M, uint32_t *copy_src, uint64_t *interp_dst,
                                   uint64_t *interp_ptr, uint32_t *interp_col, double *interp_w,
                                   uint64_t *zip_src)
{
    if (!M) return DGB_ERR_INVALID;
    if (copy_src) memcpy(copy_src, M->copy_src.data(), M->copy_src.size() * 4);
    if (interp_dst) memcpy(interp_dst, M->interp_dst.data(), M->interp_dst.size() * 8);
    if (interp_ptr) memcpy(interp_ptr, M->interp_ptr.data(), M->interp_ptr.size() * 8);
    if (interp_col) memcpy(interp_col, M->interp_col.data(), M->interp_col.size() * 4);
    if (interp_w) memcpy(interp_w, M->interp_w.data(), M->interp_w.size() * 8);
    if (zip_src) memcpy(zip_src, M->zip_src.data(), M->zip_src.size() * 8);
    return DGB_OK;
}

}  // extern "C"
