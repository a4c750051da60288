/*
 * dendro_gb300_bssn.hpp — the reference's C++ entry points for the BSSN
 * right-hand side over the C ABI (dendro_gb300.h): bssnRHS and bssnrhs with
 * the reference's array, block and offset arguments, plus what the library
 * needs that the reference keeps in globals (the bssn:: parameters as a
 * dgb_bssn_params, the octree-to-domain map, a plan cache and the
 * precision).  A solver's call site changes by those arguments (the branch
 * INTEGRATION.md shows); the stencil binding is chosen by
 * dgb_bssn_params::fd_order: 4 for the BSSN_GR solver
 * (BSSN_GR/include/rhs.h:23-37), 6 for the QuadGrav 6th-order binding.
 *
 * Header-only and templated on the caller's block type, so it compiles in
 * the reference's build against ot::Block (include/block.h) without this
 * library knowing the octree types.  The block type must provide what
 * bssnRHS reads (BSSN_GR/src/rhs.cpp:45-62): getOffset(),
 * getAllocationSz{X,Y,Z}(), getBlkNodeFlag(), computeDx/Dy/Dz(pt_min, pt_max)
 * and getBlockNode().{min,max}{X,Y,Z}().  The octree-to-domain map
 * GRIDX_TO_X (BSSN_GR/include/grDef.h:13-15) is passed in as a callable.
 *
 * Errors: the reference's functions return void and exit on failure; these
 * return the dgb_status of the first failing call instead.
 */
#pragma once
#include <vector>

#include "dendro_gb300.h"

namespace dgb_bssn {

/* Per-block descriptor exactly as bssnRHS derives it
 * (BSSN_GR/src/rhs.cpp:45-62): ptmin = GRIDX_TO_X(minX) - 3 dx,
 * ptmax = GRIDX_TO_X(maxX) + 3 dx, per axis. */
template <class Block, class Point, class GridToDomain>
dgb_block_desc describe_block(const Block &blk, const Point &pt_min, const Point &pt_max,
                              GridToDomain grid_to_domain)
{
    dgb_block_desc d;
    d.offset = blk.getOffset();
    d.sz[0] = blk.getAllocationSzX();
    d.sz[1] = blk.getAllocationSzY();
    d.sz[2] = blk.getAllocationSzZ();
    d.bflag = blk.getBlkNodeFlag();
    const double dx = blk.computeDx(pt_min, pt_max);
    const double dy = blk.computeDy(pt_min, pt_max);
    const double dz = blk.computeDz(pt_min, pt_max);
    const auto &node = blk.getBlockNode();
    d.ptmin[0] = grid_to_domain(0, node.minX()) - 3 * dx;
    d.ptmin[1] = grid_to_domain(1, node.minY()) - 3 * dy;
    d.ptmin[2] = grid_to_domain(2, node.minZ()) - 3 * dz;
    d.ptmax[0] = grid_to_domain(0, node.maxX()) + 3 * dx;
    d.ptmax[1] = grid_to_domain(1, node.maxY()) + 3 * dy;
    d.ptmax[2] = grid_to_domain(2, node.maxZ()) + 3 * dz;
    return d;
}

/* The bssn:: globals the RHS reads (BSSN_GR/include/parameters.h), and the
 * stencil binding of the solver being replaced: fd_order 4 for BSSN_GR's own
 * (deriv42, upwinded deriv42adv), 6 for QuadGrav's (deriv64). */
inline dgb_bssn_params params(const unsigned lambda[4], const double lambda_f[2],
                              double eta_const, double eta_r0, double eta_damping_exp,
                              double ko_sigma, double chi_floor, int fd_order)
{
    dgb_bssn_params p{};
    p.fd_order = fd_order;
    p.gauge = DGB_GAUGE_ETA_CONST;
    for (int i = 0; i < 4; i++) p.lambda[i] = (double)lambda[i];
    p.lambda_f[0] = lambda_f[0];
    p.lambda_f[1] = lambda_f[1];
    p.eta_const = eta_const;
    p.eta_r0 = eta_r0;
    p.eta_damping_exp = eta_damping_exp;
    p.ko_sigma = ko_sigma;
    p.chi_floor = chi_floor;
    return p;
}

/* Drop-in for void bssnRHS(double **uzipVarsRHS, const double **uZipVars,
 * const ot::Block *blkList, unsigned int numBlocks)
 * (BSSN_GR/include/rhs.h:45, BSSN_GR/src/rhs.cpp:9-76), host arrays.
 * The plan is rebuilt when the block list changes (after a remesh); keep
 * `cache` alive across calls. */
struct PlanCache {
    dgb_plan *plan = nullptr;
    std::vector<dgb_block_desc> blocks;
    ~PlanCache()
    {
        if (plan) dgb_plan_destroy(plan);
    }
};

template <class Block, class Point, class GridToDomain>
dgb_status bssnRHS(double **unzipVarsRHS, const double **uZipVars, const Block *blkList,
                   unsigned int numBlocks, const Point &pt_min, const Point &pt_max,
                   GridToDomain grid_to_domain, const dgb_bssn_params &prm, PlanCache &cache,
                   int precision = DGB_PREC_FP64)
{
    std::vector<dgb_block_desc> d(numBlocks);
    for (unsigned b = 0; b < numBlocks; b++)
        d[b] = describe_block(blkList[b], pt_min, pt_max, grid_to_domain);
    bool same = cache.plan && cache.blocks.size() == d.size();
    for (size_t b = 0; same && b < d.size(); b++) {
        const dgb_block_desc &x = d[b], &y = cache.blocks[b];
        same = x.offset == y.offset && x.sz[0] == y.sz[0] && x.sz[1] == y.sz[1] &&
               x.sz[2] == y.sz[2] && x.bflag == y.bflag && x.ptmin[0] == y.ptmin[0] &&
               x.ptmin[1] == y.ptmin[1] && x.ptmin[2] == y.ptmin[2] &&
               x.ptmax[0] == y.ptmax[0] && x.ptmax[1] == y.ptmax[1] && x.ptmax[2] == y.ptmax[2];
    }
    if (!same) {
        if (cache.plan) dgb_plan_destroy(cache.plan);
        cache.plan = nullptr;
        dgb_status s = dgb_plan_create(d.data(), d.size(), &prm, &cache.plan);
        if (s != DGB_OK) return s;
        cache.blocks = d;
    }
    return dgb_bssn_rhs_host(cache.plan, unzipVarsRHS, uZipVars, precision);
}

/* Drop-in for void bssnrhs(double **unzipVarsRHS, const double **uZipVars,
 * const unsigned int &offset, const double *pmin, const double *pmax,
 * const unsigned int *sz, const unsigned int &bflag)
 * (BSSN_GR/include/rhs.h:47-50, BSSN_GR/src/rhs.cpp:86-392), host arrays. */
inline dgb_status bssnrhs(double **unzipVarsRHS, const double **uZipVars,
                          const unsigned int &offset, const double *pmin, const double *pmax,
                          const unsigned int *sz, const unsigned int &bflag,
                          const dgb_bssn_params &prm, int precision = DGB_PREC_FP64)
{
    const uint32_t s3[3] = {sz[0], sz[1], sz[2]};
    return dgb_bssnrhs_block_host(unzipVarsRHS, uZipVars, offset, pmin, pmax, s3, bflag, &prm,
                                  precision);
}

}  // namespace dgb_bssn
