// Test infrastructure only: a C harness around the reference's own octree
// mesh (ot::Mesh, src/mesh.cpp + include/mesh.tcc), compiled from the
// reference's sources where they lie by oracle/Makefile.ref against the
// single-rank MPI stand-in and the dgesv_ of oracle/ref_mesh_shim/.  It builds
// the reference mesh from a leaf list and hands back what pins this project's
// mesh: the block list of performBlocksSetup (src/mesh.cpp:8640-8790), the
// element order, the coordinates of the CG nodes, Mesh::unzip
// (include/mesh.tcc:8693) and Mesh::zip (include/mesh.tcc:3775-3822) of
// caller-given vectors, and WaveletEl::compute_wavelets_3D
// (src/waveletRefEl.cpp:92-271) on caller-given patches.  Nothing here is
// used by the product library.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "hcurvedata.h"
#include "mesh.h"
#include "meshUtils.h"
#include "refel.h"
#include "waveletRefEl.h"

namespace {
ot::Mesh *g_mesh = nullptr;
RefElement *g_refel = nullptr;
wavelet::WaveletEl *g_wel = nullptr;
unsigned g_order = 0;
bool g_hcurve = false;
}  // namespace

extern "C" {

// Builds the reference mesh from n leaves (anchor xyz in octree units of
// max_depth, level) that already form a complete, 2:1-balanced octree:
// sorted in the reference's space-filling-curve order (TreeNode::operator<,
// Hilbert) and handed to the ot::Mesh constructor (src/mesh.cpp:283) with
// block set-up on, as ot::createMesh does after its balancing
// (src/meshUtils.cpp:120).
int refmesh_build(const uint32_t *xyz, const uint8_t *lev, uint64_t n, unsigned max_depth, unsigned order)
{
    if (!g_hcurve) {
        _InitializeHcurve(3);
        g_hcurve = true;
    }
    m_uiMaxDepth = max_depth;
    delete g_mesh;
    g_mesh = nullptr;
    std::vector<ot::TreeNode> oct;
    oct.reserve(n);
    for (uint64_t i = 0; i < n; i++)
        oct.push_back(ot::TreeNode(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], lev[i], 3, max_depth));
    std::sort(oct.begin(), oct.end());
    g_mesh = new ot::Mesh(oct, 1, order, MPI_COMM_WORLD, true, ot::SM_TYPE::FDM, DENDRO_DEFAULT_GRAIN_SZ,
                          DENDRO_DEFAULT_LB_TOL, DENDRO_DEFAULT_SF_K);
    return g_mesh ? 0 : 1;
}

void refmesh_destroy(void)
{
    delete g_mesh;
    g_mesh = nullptr;
}

// [0] all elements, [1] blocks, [2] unzipped size, [3] CG vector size,
// [4,5] local node range, [6,7] local element range
int refmesh_sizes(uint64_t *out)
{
    if (!g_mesh) return 1;
    out[0] = g_mesh->getAllElements().size();
    out[1] = g_mesh->getLocalBlockList().size();
    out[2] = g_mesh->getDegOfFreedomUnZip();
    out[3] = g_mesh->getDegOfFreedom();
    out[4] = g_mesh->getNodeLocalBegin();
    out[5] = g_mesh->getNodeLocalEnd();
    out[6] = g_mesh->getElementLocalBegin();
    out[7] = g_mesh->getElementLocalEnd();
    return 0;
}

// Per block, 12 values: block node x, y, z, level; regular-grid level;
// sizes x, y, z; offset; boundary flag (face bits); element range.
int refmesh_blocks(int64_t *out)
{
    if (!g_mesh) return 1;
    const std::vector<ot::Block> &bl = g_mesh->getLocalBlockList();
    for (size_t b = 0; b < bl.size(); b++) {
        const ot::TreeNode nd = bl[b].getBlockNode();
        int64_t *o = out + 12 * b;
        o[0] = nd.getX();
        o[1] = nd.getY();
        o[2] = nd.getZ();
        o[3] = nd.getLevel();
        o[4] = bl[b].getRegularGridLev();
        o[5] = bl[b].getAllocationSzX();
        o[6] = bl[b].getAllocationSzY();
        o[7] = bl[b].getAllocationSzZ();
        o[8] = bl[b].getOffset();
        o[9] = bl[b].getBlkNodeFlag();
        o[10] = bl[b].getLocalElementBegin();
        o[11] = bl[b].getLocalElementEnd();
    }
    return 0;
}

// Per element (all elements, in the mesh's order): x, y, z, level.
int refmesh_elements(uint32_t *out)
{
    if (!g_mesh) return 1;
    const std::vector<ot::TreeNode> &el = g_mesh->getAllElements();
    for (size_t e = 0; e < el.size(); e++) {
        out[4 * e] = el[e].getX();
        out[4 * e + 1] = el[e].getY();
        out[4 * e + 2] = el[e].getZ();
        out[4 * e + 3] = el[e].getLevel();
    }
    return 0;
}

// Coordinates (octree units) of every CG node as Mesh::createVector(func)
// evaluates them (include/mesh.tcc:124-170); NaN where it writes nothing.
int refmesh_cg_coords(double *xyz)
{
    if (!g_mesh) return 1;
    const size_t n = g_mesh->getDegOfFreedom();
    for (int a = 0; a < 3; a++) {
        double *v = g_mesh->createVector<double>([a](double x, double y, double z) {
            return a == 0 ? x : a == 1 ? y : z;
        });
        for (size_t i = 0; i < n; i++) xyz[3 * i + a] = NAN;
        for (size_t i = g_mesh->getNodeLocalBegin(); i < g_mesh->getNodeLocalEnd(); i++) xyz[3 * i + a] = v[i];
        delete[] v;
    }
    return 0;
}

// Mesh::unzip of one CG vector (size getDegOfFreedom) into uz (size
// getDegOfFreedomUnZip); uz keeps what the caller put where unzip writes nothing.
int refmesh_unzip(const double *cg, double *uz)
{
    if (!g_mesh) return 1;
    g_mesh->unzip(cg, uz, 1);
    return 0;
}

// Mesh::zip of one unzipped vector into the CG vector cg.
int refmesh_zip(const double *uz, double *cg)
{
    if (!g_mesh) return 1;
    g_mesh->zip(uz, cg);
    return 0;
}

// Per CG node, the element whose block Mesh::zip reads it from: the element
// e with E2N_DG[e, node] / NpE == e (include/mesh.tcc:3805-3807); -1 if none.
int refmesh_zip_owner(int64_t *owner)
{
    if (!g_mesh) return 1;
    const std::vector<unsigned int> &cg = g_mesh->getE2NMapping();
    const std::vector<unsigned int> &dg = g_mesh->getE2NMapping_DG();
    const size_t npe = cg.size() / g_mesh->getAllElements().size();
    for (size_t i = 0; i < g_mesh->getDegOfFreedom(); i++) owner[i] = -1;
    for (size_t e = g_mesh->getElementLocalBegin(); e < g_mesh->getElementLocalEnd(); e++)
        for (size_t k = 0; k < npe; k++)
            if (dg[e * npe + k] / npe == e) owner[cg[e * npe + k]] = (int64_t)e;
    return 0;
}

// Per local element, in the order Mesh::isReMeshUnzip visits them (blocks,
// then each block's elements, include/mesh.tcc:2066-2085): its index, its
// (2p+1)^3 padded patch of the unzipped vector uz from
// getUnzipElementalNodalValues (include/mesh.tcc:9136-9176) into patches
// (13^3 doubles each at p = 6, x fastest; NULL skips them) and
// isBoundaryOctant (include/mesh.h:1482-1486) into bdy.
int refmesh_element_patches(const double *uz, int64_t *elem, double *patches, uint8_t *bdy)
{
    if (!g_mesh) return 1;
    const std::vector<ot::Block> &bl = g_mesh->getLocalBlockList();
    const unsigned p = g_mesh->getElementOrder();
    const size_t np = (size_t)(2 * p + 1) * (2 * p + 1) * (2 * p + 1);
    size_t q = 0;
    for (unsigned b = 0; b < bl.size(); b++)
        for (unsigned e = bl[b].getLocalElementBegin(); e < bl[b].getLocalElementEnd(); e++, q++) {
            elem[q] = e;
            if (patches) g_mesh->getUnzipElementalNodalValues(uz, b, e, patches + q * np, true);
            bdy[q] = g_mesh->isBoundaryOctant(e) ? 1 : 0;
        }
    return 0;
}

// WaveletEl::compute_wavelets_3D on one padded element patch (side
// 2*order+1 points per axis, as Mesh::isReMeshUnzip passes it):
// wc receives the wavelet coefficients (count returned in *nwc).
int refmesh_wavelets(unsigned order, const double *patch, const unsigned *isz, int is_bdy, double *wc, unsigned *nwc)
{
    if (!g_refel || g_order != order) {
        delete g_wel;
        delete g_refel;
        g_refel = new RefElement(3, order);
        g_wel = new wavelet::WaveletEl(g_refel);
        g_order = order;
    }
    std::vector<double> w;
    g_wel->compute_wavelets_3D(patch, isz, w, is_bdy != 0);
    for (size_t i = 0; i < w.size(); i++) wc[i] = w[i];
    *nwc = (unsigned)w.size();
    return 0;
}

}  // extern "C"
