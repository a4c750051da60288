// Host-side octree mesh for the full-step path: a 2:1-balanced octree
// refined around the punctures, its regular blocks, the continuous-Galerkin
// node numbering (the "zipped" vector) and the unzip / zip operators.
//
// What it reproduces of the reference's ot::Mesh (src/mesh.cpp, include/mesh.tcc);
// the oracle build of that mesh gives the same blocks, offsets, CG numbering
// and zip, and the same unzip to rounding, on these octrees:
//   octree + 2:1 balance        ot::Mesh construction (src/mesh.cpp:283),
//                               balance across faces, edges and corners
//   element order               the reference's Hilbert curve (TreeNode::operator<)
//   blocks                      octree2BlockDecomposition (src/octUtils.cpp:556-741)
//                               / performBlocksSetup (src/mesh.cpp:8640-8790):
//                               regular-grid levels passed down the octree in curve
//                               order, side p*2^k + 1 + 6 (src/block.cpp:50),
//                               offsets = exclusive prefix sum (src/mesh.cpp:8667-8672),
//                               bflag = domain faces touched (src/mesh.cpp:8701-8738);
//                               max_block_refine >= 0 selects maximal aligned cubes of
//                               at most 2^max_block_refine leaves per side instead
//   zipped vector               one value per independent element node (a node
//   (Mesh::buildE2NMap,         position is independent when it lies on the node
//   src/mesh.cpp:3895-3960)     lattice of every leaf whose closure contains it);
//                               owner = the coarsest element holding it, first in
//                               element order on ties; CG order = (owner, place in
//                               the owner, x fastest)
//   Mesh::unzip                 every padded point inside the domain gets the mesh
//   (include/mesh.tcc:7436-8690) field at its position: an independent node's value,
//                               or the degree-p Lagrange interpolant of the coarsest
//                               leaf containing it, evaluated from that leaf's nodal
//                               values, whose hanging nodes are interpolated the same
//                               way from coarser leaves (getElementNodalValues,
//                               mesh.tcc:2467).  This is the reference's element copy,
//                               same-level padding copy, coarser-neighbour
//                               parent->child interpolation (FEM/include/refel.h:249-296),
//                               finer-neighbour child->parent injection
//                               (mesh.tcc:7399-7433) and edge/corner padding, as one rule.
//   Mesh::zip                   every independent node takes the value at its
//   (include/mesh.tcc:3775-3822) position in its owner's block.
//
// Operator encoding (see dgb_unzip_plan_create): a node reference is a 64-bit
// word; bit 63 clear: copy independent node (low 32 bits); bit 63 set:
// interpolate from source leaf (bits 12..42) at local position codes
// (bits 0..11, 4 bits per axis, code = 2 * xi, xi in [0, 6]).  Source leaves
// hold their 343 nodal values and are filled coarsest level first.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <string>
#include <unordered_map>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../../include/dendro_gb300.h"

namespace {

constexpr int P = 6;  // element order
constexpr int NPE = (P + 1) * (P + 1) * (P + 1);
constexpr uint64_t kInterp = 1ull << 63;
constexpr uint64_t kNone = ~0ull;

struct Leaf {
    uint32_t a[3];  // anchor in node-lattice units
    int lev;
};

inline uint64_t key(int lev, uint32_t x, uint32_t y, uint32_t z)
{
    return ((uint64_t)lev << 48) | ((uint64_t)x << 32) | ((uint64_t)y << 16) | (uint64_t)z;
}
inline uint64_t pkey(uint64_t x, uint64_t y, uint64_t z) { return (x << 32) | (y << 16) | z; }

// The reference's space-filling curve (Hilbert ordering, on by default:
// CMakeLists.txt:32; tables in src/hcurvedata.cpp, used by
// TreeNode::operator< and octree2BlockDecomposition, src/octUtils.cpp:556).
// A state of the curve is a symmetry of the cube (an axis permutation with
// reflections) applied to the base visiting order of the eight children;
// child c = x | y << 1 | z << 2.  The base order and the symmetry each visited
// child takes relative to its parent define the reference's particular curve:
// the 24 states they generate give the same visiting orders and transitions
// as the reference's tables (a test builds both and compares them).
struct CubeSym {
    uint8_t perm[3], flip[3];  // bit a of the image = bit perm[a] of the input ^ flip[a]
    int apply(int c) const
    {
        int w = 0;
        for (int a = 0; a < 3; a++) w |= (((c >> perm[a]) & 1) ^ flip[a]) << a;
        return w;
    }
    CubeSym then(const CubeSym &inner) const  // this o inner
    {
        CubeSym r;
        for (int a = 0; a < 3; a++) {
            r.perm[a] = inner.perm[perm[a]];
            r.flip[a] = (uint8_t)(inner.flip[perm[a]] ^ flip[a]);
        }
        return r;
    }
    bool operator==(const CubeSym &o) const { return memcmp(this, &o, sizeof o) == 0; }
};

struct HilbertCurve {
    static constexpr int kBase[8] = {0, 2, 3, 1, 5, 7, 6, 4};
    std::vector<CubeSym> state;
    std::vector<std::array<uint8_t, 8>> order;  // [state][i] = child visited i-th
    std::vector<std::array<uint8_t, 8>> pos;    // [state][child] = its place in the visit
    std::vector<std::array<uint8_t, 8>> next;   // [state][child] = the child's state
    HilbertCurve()
    {
        const CubeSym visit[8] = {{{0, 2, 1}, {0, 0, 0}}, {{2, 1, 0}, {0, 0, 0}}, {{0, 1, 2}, {0, 0, 0}},
                                  {{2, 0, 1}, {0, 1, 1}}, {{2, 0, 1}, {1, 1, 0}}, {{0, 1, 2}, {0, 0, 0}},
                                  {{2, 1, 0}, {1, 0, 1}}, {{0, 2, 1}, {0, 1, 1}}};
        state.push_back(CubeSym{{0, 1, 2}, {0, 0, 0}});
        for (size_t s = 0; s < state.size(); s++) {
            std::array<uint8_t, 8> o, p, n;
            for (int i = 0; i < 8; i++) {
                const int c = state[s].apply(kBase[i]);
                o[i] = (uint8_t)c;
                p[c] = (uint8_t)i;
                const CubeSym cs = state[s].then(visit[i]);
                size_t id = 0;
                while (id < state.size() && !(state[id] == cs)) id++;
                if (id == state.size()) state.push_back(cs);
                n[c] = (uint8_t)id;
            }
            order.push_back(o);
            pos.push_back(p);
            next.push_back(n);
        }
    }
    // Key of the octant at level lev whose anchor has integer coordinates a
    // (units of the finest level D): three bits per level from the root,
    // left-aligned to D levels, so that disjoint octants sort in curve order.
    uint64_t key(const uint32_t a[3], int lev, int D) const
    {
        uint64_t k = 0;
        int s = 0;
        for (int l = 1; l <= lev; l++) {
            const int sh = D - l;
            const int c = (int)((a[0] >> sh) & 1u) | (int)(((a[1] >> sh) & 1u) << 1) | (int)(((a[2] >> sh) & 1u) << 2);
            k = (k << 3) | pos[s][c];
            s = next[s][c];
        }
        return k << (3 * (D - lev));
    }
};
constexpr int HilbertCurve::kBase[8];

const HilbertCurve &hilbert()
{
    static const HilbertCurve h;
    return h;
}

}  // namespace

extern "C" dgb_status dgb_mesh_hilbert_tables(uint8_t *order, uint8_t *next, int *nstates)
{
    const HilbertCurve &h = hilbert();
    if (nstates) *nstates = (int)h.state.size();
    for (size_t s = 0; s < h.state.size(); s++)
        for (int i = 0; i < 8; i++) {
            if (order) order[8 * s + i] = h.order[s][i];
            if (next) next[8 * s + i] = h.next[s][i];
        }
    return DGB_OK;
}

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
    std::vector<uint64_t> dof_keys;      // positions of the independent nodes, in CG order
    std::vector<uint64_t> own_mask;      // 6 words per leaf: the nodal points the leaf owns
    std::vector<uint64_t> first_dof;     // per leaf: CG index of its first owned node
    // unzip operator
    std::vector<uint32_t> copy_src;      // per padded point: dof, or 0xFFFFFFFF
    std::vector<uint64_t> interp_dst, interp_ref;
    std::vector<uint64_t> src_leaf;      // source leaves, by level ascending
    std::vector<uint64_t> src_refs;      // 343 refs per source leaf
    std::vector<uint64_t> level_ptr;     // source-leaf ranges per distinct level
    std::vector<uint64_t> zip_src;       // per dof: padded point it is read from

    uint32_t S(int lev) const { return (uint32_t)P << (D - lev); }  // leaf size
    uint32_t sp(int lev) const { return 1u << (D - lev); }         // node spacing

    // Leaf containing the point q + eps * dir (dir components in {-1, +1}),
    // or -1 outside the domain.  hint: a level to try first (2:1 balance keeps
    // neighbours within one level).
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
    // Coarsest leaf whose closure holds q, first in element order on ties
    // (the owner of q when it is a node); also whether q is an independent node.
    int64_t coarsest_at(const int64_t q[3], bool *independent, int hint = -1) const
    {
        int64_t best = -1;
        bool indep = true;
        for (int c = 0; c < 8; c++) {
            const int dir[3] = {(c & 1) ? 1 : -1, (c & 2) ? 1 : -1, (c & 4) ? 1 : -1};
            const int64_t e = leaf_at(q, dir, hint);
            if (e < 0) continue;
            hint = leaves[e].lev;
            if (!on_lattice(leaves[e], q)) indep = false;
            if (best < 0 || leaves[e].lev < leaves[best].lev || (leaves[e].lev == leaves[best].lev && e < best))
                best = e;
        }
        if (independent) *independent = indep;
        return best;
    }
    // CG index of the independent node q owned by leaf e: e's first index plus
    // the number of nodes e owns before q's place in it.
    int64_t dof(int64_t e, const int64_t q[3]) const
    {
        const Leaf &L = leaves[e];
        const int64_t s = sp(L.lev);
        int loc[3];
        for (int a = 0; a < 3; a++) {
            const int64_t d = q[a] - (int64_t)L.a[a];
            if (d < 0 || d % s != 0 || d / s > P) return -1;
            loc[a] = (int)(d / s);
        }
        const int l = loc[0] + (P + 1) * (loc[1] + (P + 1) * loc[2]);
        const uint64_t *m = &own_mask[6 * e];
        if (!((m[l >> 6] >> (l & 63)) & 1)) return -1;
        uint64_t before = 0;
        for (int w = 0; w < (l >> 6); w++) before += (uint64_t)__builtin_popcountll(m[w]);
        if (l & 63) before += (uint64_t)__builtin_popcountll(m[l >> 6] & ((1ull << (l & 63)) - 1));
        return (int64_t)(first_dof[e] + before);
    }
    // Reference for the field at lattice point q (kNone outside the domain);
    // interpolation references carry the LEAF index until sources are numbered.
    uint64_t resolve(const int64_t q[3], int hint) const
    {
        bool indep = false;
        const int64_t e = coarsest_at(q, &indep, hint);
        if (e < 0) return kNone;
        if (indep) {
            const int64_t d = dof(e, q);
            return d < 0 ? kNone : (uint64_t)d;
        }
        const Leaf &L = leaves[e];
        const int64_t s = sp(L.lev);
        uint64_t codes = 0;
        for (int a = 0; a < 3; a++) {
            const int64_t d2 = 2 * (q[a] - (int64_t)L.a[a]);
            if (d2 % s != 0) return kNone;  // not on the half lattice: 2:1 balance violated
            codes |= (uint64_t)(d2 / s) << (4 * a);
        }
        return kInterp | ((uint64_t)e << 12) | codes;
    }
};

namespace {

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

void children(const dgb_mesh &M, const Leaf &o, std::vector<Leaf> &out)
{
    const uint32_t h = M.S(o.lev + 1);
    for (int c = 0; c < 8; c++)
        out.push_back(Leaf{{o.a[0] + ((c & 1) ? h : 0), o.a[1] + ((c & 2) ? h : 0),
                            o.a[2] + ((c & 4) ? h : 0)}, o.lev + 1});
}

}  // namespace

extern "C" {

dgb_status dgb_mesh_create(const dgb_mesh_params *prm, dgb_mesh **out)
{
    if (!prm || !out) return DGB_ERR_INVALID;
    *out = nullptr;
    if (prm->ele_order != P || prm->max_level < prm->min_level || prm->max_level > 12 ||
        prm->min_level < 1 || prm->num_punctures < 0 || prm->num_punctures > 4 ||
        prm->max_block_refine < -1 || prm->max_block_refine > 3 ||
        (prm->octree_depth != 0 && (prm->octree_depth < prm->max_level + 3 || prm->octree_depth > 30)))
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
        if (o.lev < target_level(*M, o))
            children(*M, o, work);
        else
            leaves.push_back(o);
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
        std::vector<uint8_t> refine(leaves.size(), 0);
        int any = 0;
#pragma omp parallel for schedule(dynamic, 1024) reduction(| : any)
        for (long long i = 0; i < (long long)leaves.size(); i++) {
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
                            __atomic_store_n(&refine[nb], (uint8_t)1, __ATOMIC_RELAXED);
                            any = 1;
                        }
                    }
        }
        if (!any) break;
        std::vector<Leaf> next;
        next.reserve(leaves.size() + 8);
        for (size_t i = 0; i < leaves.size(); i++) {
            if (refine[i])
                children(*M, leaves[i], next);
            else
                next.push_back(leaves[i]);
        }
        leaves.swap(next);
    }
    // ---- element order: the reference's space-filling curve (its
    // m_uiAllElements order, so leaf indices are element indices)
    {
        const HilbertCurve &hc = hilbert();
        std::vector<std::pair<uint64_t, uint32_t>> hk(leaves.size());
        for (size_t i = 0; i < leaves.size(); i++) {
            const uint32_t a[3] = {leaves[i].a[0] / P, leaves[i].a[1] / P, leaves[i].a[2] / P};
            hk[i] = {hc.key(a, leaves[i].lev, M->D), (uint32_t)i};
        }
        std::sort(hk.begin(), hk.end());
        std::vector<Leaf> sorted(leaves.size());
        for (size_t i = 0; i < leaves.size(); i++) sorted[i] = leaves[hk[i].second];
        leaves.swap(sorted);
    }
    rebuild_index();

    // ---- blocks
    struct BlockNode {
        uint32_t a[3];  // anchor, lattice units
        int node_lev, reg_lev;
    };
    std::vector<BlockNode> bnodes;
    if (prm->max_block_refine < 0) {
        // octree2BlockDecomposition (src/octUtils.cpp:556-741) with no tags,
        // coarsest block level 0 (src/mesh.cpp:290), its constants
        // OCT2BLK_DECOMP_LEV_GAP = 0 and fill ratio 0.5 (include/octUtils.h:39-40)
        // and the octree depth m_uiMaxDepth of the reference's coordinates:
        // a node whose leaves all have its regular-grid level r is a block of
        // 2^(r - node level) leaves per side; otherwise each child is examined in
        // curve order with level r if it holds a leaf of level r, else r + 1.
        // The root starts at the coarsest leaf level.  Visiting the children in
        // curve order lists the blocks in the order the reference's stack and
        // final reversal leave them.
        const HilbertCurve &hc = hilbert();
        const int md = prm->octree_depth > 0 ? prm->octree_depth : M->D + 4;  // m_uiMaxDepth
        int dmin = M->D, dmax = 0;
        for (const Leaf &l : leaves) {
            dmin = std::min(dmin, l.lev);
            dmax = std::max(dmax, l.lev);
        }
        struct Item {
            uint32_t a[3];
            int lev, reg, rot;
            size_t b, e;  // leaf range
        };
        std::vector<Item> stack{Item{{0, 0, 0}, 0, dmin, 0, 0, leaves.size()}};
        while (!stack.empty()) {
            const Item it = stack.back();
            stack.pop_back();
            bool uniform = true;
            for (size_t i = it.b; i < it.e && uniform; i++) uniform = leaves[i].lev == it.reg;
            // the volume test octVolume == blockVolume (src/octUtils.cpp:620-662)
            // in the reference's arithmetic: each term is 1u << 3*(maxDepth - level)
            // in 32-bit unsigned int, a shift that only keeps its count mod 32
            // (the x86-64 and AArch64 shift instructions), summed in 128 bits; so
            // a node of 2^32 octree units or more is never accepted whole
            if (uniform && it.lev != it.reg) {
                const unsigned __int128 count = (unsigned __int128)1 << (3 * (it.reg - it.lev));
                const uint32_t vol_leaf = 1u << ((3 * (md - it.reg)) & 31);
                const uint32_t vol_node = 1u << ((3 * (md - it.lev)) & 31);
                uniform = count * vol_leaf == (unsigned __int128)vol_node;
            }
            if (uniform) {
                bnodes.push_back(BlockNode{{it.a[0], it.a[1], it.a[2]}, it.lev, it.reg});
                continue;
            }
            // children of the node: contiguous leaf ranges in curve order
            const uint32_t half = M->S(it.lev + 1);
            Item kids[8];
            int nk = 0;
            size_t i = it.b;
            for (int v = 0; v < 8; v++) {
                const int c = hc.order[it.rot][v];
                Item k;
                for (int a = 0; a < 3; a++) k.a[a] = it.a[a] + (((c >> a) & 1) ? half : 0);
                k.lev = it.lev + 1;
                k.rot = hc.next[it.rot][c];
                k.b = i;
                bool has_reg = false;
                while (i < it.e) {
                    const Leaf &l = leaves[i];
                    bool in = true;
                    for (int a = 0; a < 3; a++) in = in && l.a[a] >= k.a[a] && l.a[a] < k.a[a] + half;
                    if (!in) break;
                    has_reg = has_reg || l.lev == it.reg;
                    i++;
                }
                k.e = i;
                if (k.e == k.b) continue;
                k.reg = has_reg ? it.reg : it.reg + 1;
                if (k.reg > dmax) continue;
                kids[nk++] = k;
            }
            if (i != it.e) {  // the leaves are not in curve order: cannot happen
                delete M;
                return DGB_ERR_INVALID;
            }
            for (int v = nk - 1; v >= 0; v--) stack.push_back(kids[v]);  // first child on top
        }
    } else {
        // maximal aligned cubes of 2^k leaves of one level (k <= max_block_refine),
        // found in Morton order and then listed in curve order
        std::vector<uint32_t> morder(leaves.size());
        for (size_t i = 0; i < leaves.size(); i++) morder[i] = (uint32_t)i;
        auto morton = [&](const Leaf &l) {
            uint64_t m = 0;
            for (int b = 15; b >= 0; b--)
                for (int a = 2; a >= 0; a--) m = (m << 1) | ((l.a[a] / P) >> b & 1u);
            return m;
        };
        std::sort(morder.begin(), morder.end(),
                  [&](uint32_t x, uint32_t y) { return morton(leaves[x]) < morton(leaves[y]); });
        std::vector<char> used(leaves.size(), 0);
        const int kmax = prm->max_block_refine;
        std::vector<std::pair<uint64_t, BlockNode>> found;
        for (uint32_t i : morder) {
            if (used[i]) continue;
            const Leaf e = leaves[i];
            int kbest = 0;
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
                    break;
                }
            }
            const uint32_t s = M->S(e.lev), m = 1u << kbest;
            for (uint32_t z = 0; z < m; z++)
                for (uint32_t y = 0; y < m; y++)
                    for (uint32_t x = 0; x < m; x++)
                        used[M->leaf_of[key(e.lev, e.a[0] + x * s, e.a[1] + y * s, e.a[2] + z * s)]] = 1;
            const uint32_t a[3] = {e.a[0] / P, e.a[1] / P, e.a[2] / P};
            found.push_back({hilbert().key(a, e.lev - kbest, M->D),
                             BlockNode{{e.a[0], e.a[1], e.a[2]}, e.lev - kbest, e.lev}});
        }
        std::sort(found.begin(), found.end(),
                  [](const std::pair<uint64_t, BlockNode> &x, const std::pair<uint64_t, BlockNode> &y) {
                      return x.first < y.first;
                  });
        for (auto &f : found) bnodes.push_back(f.second);
    }
    // block descriptors (src/block.cpp:38-55), offsets = exclusive prefix sum
    // (src/mesh.cpp:8661-8675), face flags (src/mesh.cpp:8701-8738)
    std::vector<uint32_t> leaf_block(leaves.size(), 0xFFFFFFFFu);
    uint64_t off = 0;
    for (size_t bi = 0; bi < bnodes.size(); bi++) {
        const BlockNode &bn = bnodes[bi];
        const uint32_t m = 1u << (bn.reg_lev - bn.node_lev);
        const uint32_t s = M->S(bn.reg_lev);
        dgb_block_desc b;
        memset(&b, 0, sizeof b);
        const uint32_t side = (uint32_t)P * m + 1 + 6;
        const double h = M->sp(bn.reg_lev) * M->unit;
        for (int a = 0; a < 3; a++) {
            b.sz[a] = side;
            const double x0 = prm->domain_min[a] + bn.a[a] * M->unit;
            b.ptmin[a] = x0 - 3 * h;
            b.ptmax[a] = x0 + (double)(P * m) * h + 3 * h;
            if (bn.a[a] == 0) b.bflag |= 1u << (2 * a);
            if (bn.a[a] + s * m == M->N) b.bflag |= 1u << (2 * a + 1);
        }
        b.offset = off;
        off += (uint64_t)side * side * side;
        M->blocks.push_back(b);
        M->block_lev.push_back(bn.reg_lev);
        M->block_anchor.insert(M->block_anchor.end(), bn.a, bn.a + 3);
        for (uint32_t z = 0; z < m; z++)
            for (uint32_t y = 0; y < m; y++)
                for (uint32_t x = 0; x < m; x++) {
                    auto it = M->leaf_of.find(key(bn.reg_lev, bn.a[0] + x * s, bn.a[1] + y * s, bn.a[2] + z * s));
                    if (it == M->leaf_of.end() || leaf_block[it->second] != 0xFFFFFFFFu) {
                        delete M;
                        return DGB_ERR_INVALID;
                    }
                    leaf_block[it->second] = (uint32_t)bi;
                }
    }
    for (uint32_t lb : leaf_block)
        if (lb == 0xFFFFFFFFu) {
            delete M;
            return DGB_ERR_INVALID;
        }

    // ---- independent nodes and their numbering (Mesh::buildE2NMap,
    // src/mesh.cpp:3895-3960): a node is owned by the coarsest element that
    // has it as a nodal point, the one first in element order on ties; the CG
    // vector lists the nodes by owner, then by the node's place in the owner
    // (x fastest).  Per leaf: a 343-bit mask of the nodes it owns and the index
    // of its first one.
    M->own_mask.assign(leaves.size() * 6, 0);
    M->first_dof.assign(leaves.size() + 1, 0);
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)leaves.size(); i++) {
        const Leaf &e = leaves[i];
        const int64_t s = M->sp(e.lev);
        uint64_t *mask = &M->own_mask[6 * i];
        uint64_t cnt = 0;
        for (int k = 0; k <= P; k++)
            for (int j = 0; j <= P; j++)
                for (int ii = 0; ii <= P; ii++) {
                    bool mine = true;
                    if (ii == 0 || ii == P || j == 0 || j == P || k == 0 || k == P) {
                        const int64_t q[3] = {(int64_t)e.a[0] + s * ii, (int64_t)e.a[1] + s * j,
                                              (int64_t)e.a[2] + s * k};
                        bool indep = true;
                        mine = M->coarsest_at(q, &indep, e.lev) == (int64_t)i && indep;
                    }
                    if (mine) {
                        const int l = ii + (P + 1) * (j + (P + 1) * k);
                        mask[l >> 6] |= 1ull << (l & 63);
                        cnt++;
                    }
                }
        M->first_dof[i + 1] = cnt;
    }
    for (size_t i = 0; i < leaves.size(); i++) M->first_dof[i + 1] += M->first_dof[i];
    const uint64_t ndof = M->first_dof[leaves.size()];
    if (ndof >= 0xFFFFFFFFull) {
        delete M;
        return DGB_ERR_INVALID;
    }
    // positions and zip sources (Mesh::zip, include/mesh.tcc:3775-3822: a node
    // is read from its owner's block)
    M->dof_keys.resize(ndof);
    M->zip_src.resize(ndof);
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)leaves.size(); i++) {
        const Leaf &e = leaves[i];
        const int64_t s = M->sp(e.lev);
        const uint64_t *mask = &M->own_mask[6 * i];
        const uint32_t b = leaf_block[i];
        const dgb_block_desc &B = M->blocks[b];
        const uint32_t *A = &M->block_anchor[3 * b];
        const uint64_t n = B.sz[0];
        uint64_t d = M->first_dof[i];
        for (int l = 0; l < NPE; l++) {
            if (!((mask[l >> 6] >> (l & 63)) & 1)) continue;
            const int ii = l % (P + 1), j = (l / (P + 1)) % (P + 1), k = l / ((P + 1) * (P + 1));
            const uint64_t q[3] = {e.a[0] + (uint64_t)s * ii, e.a[1] + (uint64_t)s * j, e.a[2] + (uint64_t)s * k};
            M->dof_keys[d] = pkey(q[0], q[1], q[2]);
            uint64_t p[3];
            for (int a = 0; a < 3; a++) p[a] = (q[a] - A[a]) / (uint64_t)s + 3;
            M->zip_src[d] = B.offset + p[0] + n * (p[1] + n * p[2]);
            d++;
        }
    }

    // ---- padded points: copy or interpolation reference (parallel over blocks)
    const uint32_t SENT = 0xFFFFFFFFu;
    M->copy_src.assign(off, SENT);
    std::vector<uint8_t> is_src(leaves.size(), 0);
    std::vector<std::vector<std::pair<uint64_t, uint64_t>>> rows_part;
    int ntr = 1;
#ifdef _OPENMP
    ntr = omp_get_max_threads();
#endif
    rows_part.resize(ntr);
    std::atomic<int> bad{0};
#pragma omp parallel
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
#pragma omp for schedule(dynamic, 4)
        for (long long b = 0; b < (long long)M->blocks.size(); b++) {
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
                        const uint64_t r = M->resolve(q, lev);
                        if (r == kNone) {
                            bad = 1;
                        } else if (r & kInterp) {
                            rows_part[t].push_back({dst, r});
                            __atomic_store_n(&is_src[(r >> 12) & 0x7FFFFFFFull], (uint8_t)1, __ATOMIC_RELAXED);
                        } else {
                            M->copy_src[dst] = (uint32_t)r;
                        }
                    }
        }
    }
    if (bad) {
        delete M;
        return DGB_ERR_INVALID;
    }
    // ---- source leaves: close under hanging-node references, finest level first
    std::vector<std::vector<uint64_t>> leaf_refs(leaves.size());
    for (int lev = M->D; lev >= 0; lev--) {
        std::vector<long long> at;
        for (size_t i = 0; i < leaves.size(); i++)
            if (is_src[i] && leaves[i].lev == lev) at.push_back((long long)i);
#pragma omp parallel for schedule(dynamic, 16)
        for (long long q2 = 0; q2 < (long long)at.size(); q2++) {
            const long long i = at[q2];
            const Leaf &e = leaves[i];
            const int64_t s = M->sp(e.lev);
            std::vector<uint64_t> refs(NPE);
            for (int k = 0; k <= P; k++)
                for (int j = 0; j <= P; j++)
                    for (int ii = 0; ii <= P; ii++) {
                        const int64_t q[3] = {(int64_t)e.a[0] + s * ii, (int64_t)e.a[1] + s * j,
                                              (int64_t)e.a[2] + s * k};
                        const uint64_t r = M->resolve(q, e.lev);
                        refs[ii + (P + 1) * (j + (P + 1) * k)] = r;
                        if (r == kNone) bad = 1;
                        else if (r & kInterp)
                            __atomic_store_n(&is_src[(r >> 12) & 0x7FFFFFFFull], (uint8_t)1, __ATOMIC_RELAXED);
                    }
            leaf_refs[i].swap(refs);
        }
    }
    if (bad) {
        delete M;
        return DGB_ERR_INVALID;
    }
    // number the sources by level ascending; remap leaf indices to source indices
    std::vector<uint64_t> src_of(leaves.size(), kNone);
    for (int lev = 0; lev <= M->D; lev++) {
        bool opened = false;
        for (size_t i = 0; i < leaves.size(); i++) {
            if (!is_src[i] || leaves[i].lev != lev) continue;
            if (!opened) {
                M->level_ptr.push_back(M->src_leaf.size());
                opened = true;
            }
            src_of[i] = M->src_leaf.size();
            M->src_leaf.push_back(i);
        }
    }
    M->level_ptr.push_back(M->src_leaf.size());
    auto remap = [&](uint64_t r) -> uint64_t {
        if (!(r & kInterp)) return r;
        const uint64_t leaf = (r >> 12) & 0x7FFFFFFFull;
        return kInterp | (src_of[leaf] << 12) | (r & 0xFFFull);
    };
    M->src_refs.resize(M->src_leaf.size() * NPE);
    for (size_t sidx = 0; sidx < M->src_leaf.size(); sidx++) {
        const auto &refs = leaf_refs[M->src_leaf[sidx]];
        for (int n = 0; n < NPE; n++) M->src_refs[sidx * NPE + n] = remap(refs[n]);
    }
    for (auto &part : rows_part) {
        for (auto &dr : part) {
            M->interp_dst.push_back(dr.first);
            M->interp_ref.push_back(remap(dr.second));
        }
        std::vector<std::pair<uint64_t, uint64_t>>().swap(part);
    }
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
    sizes[1] = M->dof_keys.size();
    sizes[2] = M->blocks.size();
    sizes[3] = M->copy_src.size();
    sizes[4] = M->interp_dst.size();
    sizes[5] = M->src_leaf.size();
    sizes[6] = M->level_ptr.size() ? M->level_ptr.size() - 1 : 0;
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
    const size_t n = M->dof_keys.size();
    for (size_t d = 0; d < n; d++) {
        const uint64_t k = M->dof_keys[d];
        const uint64_t c[3] = {k >> 32, (k >> 16) & 0xFFFF, k & 0xFFFF};
        for (int a = 0; a < 3; a++) xyz[3 * d + a] = M->prm.domain_min[a] + c[a] * M->unit;
    }
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
                                   uint64_t *interp_ref, uint64_t *src_refs, uint64_t *level_ptr,
                                   uint64_t *zip_src)
{
    if (!M) return DGB_ERR_INVALID;
    if (copy_src) memcpy(copy_src, M->copy_src.data(), M->copy_src.size() * 4);
    if (interp_dst) memcpy(interp_dst, M->interp_dst.data(), M->interp_dst.size() * 8);
    if (interp_ref) memcpy(interp_ref, M->interp_ref.data(), M->interp_ref.size() * 8);
    if (src_refs) memcpy(src_refs, M->src_refs.data(), M->src_refs.size() * 8);
    if (level_ptr) memcpy(level_ptr, M->level_ptr.data(), M->level_ptr.size() * 8);
    if (zip_src) memcpy(zip_src, M->zip_src.data(), M->zip_src.size() * 8);
    return DGB_OK;
}

dgb_status dgb_mesh_leaf_patches(const dgb_mesh *M, uint64_t *patch_base, uint32_t *block_side,
                                 uint8_t *boundary, double *corner, double *hx)
{
    if (!M) return DGB_ERR_INVALID;
    // a block of side P*m + 7 holds m^3 leaves of its level; leaf (x, y, z)
    // of the block starts at padded index P*(x, y, z)
    for (size_t b = 0; b < M->blocks.size(); b++) {
        const dgb_block_desc &d = M->blocks[b];
        const uint32_t side = d.sz[0], m = (side - 7) / P;
        const int lev = M->block_lev[b];
        const uint32_t s = M->S(lev);
        const uint32_t *anc = &M->block_anchor[3 * b];
        for (uint32_t z = 0; z < m; z++)
            for (uint32_t y = 0; y < m; y++)
                for (uint32_t x = 0; x < m; x++) {
                    const uint32_t a[3] = {anc[0] + x * s, anc[1] + y * s, anc[2] + z * s};
                    auto it = M->leaf_of.find(key(lev, a[0], a[1], a[2]));
                    if (it == M->leaf_of.end()) return DGB_ERR_INVALID;
                    const uint32_t e = it->second;
                    if (patch_base)
                        patch_base[e] = d.offset + (uint64_t)P * x +
                                        (uint64_t)side * ((uint64_t)P * y + (uint64_t)side * P * z);
                    if (block_side) block_side[e] = side;
                    bool bdy = false;
                    for (int q = 0; q < 3; q++) bdy = bdy || a[q] == 0 || a[q] + s == M->N;
                    if (boundary) boundary[e] = bdy;
                    if (corner)
                        for (int q = 0; q < 3; q++)
                            corner[3 * e + q] = M->prm.domain_min[q] + a[q] * M->unit;
                    if (hx) hx[e] = M->sp(lev) * M->unit;
                }
    }
    return DGB_OK;
}

dgb_status dgb_wavelet_tol_radial(const double *corner, uint64_t n, double tol_min, double tol_max,
                                  double r0, double r1, int use_function, double *tol)
{
    if ((n && (!corner || !tol)) || (use_function && r1 == r0)) return DGB_ERR_INVALID;
    for (uint64_t e = 0; e < n; e++) {
        if (!use_function) {
            tol[e] = tol_min;
            continue;
        }
        const double *c = corner + 3 * e;
        const double r = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        tol[e] = std::min(tol_max, std::max(tol_min, (tol_max - tol_min) / (r1 - r0) * (r - r0) + tol_min));
    }
    return DGB_OK;
}

}  // extern "C"
