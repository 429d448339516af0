/*
 * Oracle: plain-C restatement of the reference lattice-Boltzmann time step.
 *
 * TEST INFRASTRUCTURE ONLY.  Used by the tests as the checker and by the
 * benchmark as the timed CPU baseline; the product never links or calls it.
 *
 * Everything works on the reference's own data layout and numbering:
 *   f     [n_nodes][nfields][nq]  LbField  (src/lbsolver/LBfield.h:298-305)
 *   rho   [n_nodes][nfields]      ScalarField (LBfield.h:92-100)
 *   vel   [n_nodes][nd]           VectorField (LBfield.h:168-175)
 *   neigh [n_nodes][nq]           Grid::neigList_ (src/lbsolver/LBgrid.h:119, 197)
 *   types [n_nodes]               Nodes::nodeType_ (src/lbsolver/LBnodes.h:107)
 * and follows the reference algorithm literally: collide each bulk node, push
 * to the neighbours (LbField::propagateTo, LBfield.h:350-357), swap, then the
 * half-way bounce-back pass (src/lbsolver/LBhalfwaybb.h:37-71).  Arithmetic is
 * evaluated in the reference's expression order so that, compiled without FMA
 * contraction, results are bit-identical to the reference's.
 */
#ifndef BCLBM_ORACLE_H
#define BCLBM_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int nq;             /* 9 (D2Q9) or 19 (D3Q19) */
    int n_nodes;        /* N = grid.size(), node 0 is the ghost */
    const int32_t* neigh;
    const int16_t* types;
    int n_bulk;
    const int32_t* bulk;   /* findBulkNodes order */
} oracle_grid;

/* std_case step (src/std_case/main.cpp:110-145), BGK or TRT.
 * f, ftmp: two LbField(1, N) buffers (swapData exchanges their roles each step).
 * Returns 0 if the state after the last step is in f, 1 if it is in ftmp,
 * negative on invalid input.
 * rho, vel receive the moments of the last step's collision (may be NULL).
 * trt = 0: calcOmegaBGK + calcDeltaOmegaF (LBcollision.h:27-46, 194-213).
 * trt = 1: calcOmegaBGKTRT(tau, tau_anti) + calcDeltaOmegaFTRT(phi = 1)
 *          (LBcollision.h:50-75, 215-236).
 * nthreads: host threads for the node loops (results do not depend on it). */
int oracle_single_run(const oracle_grid* g, int nsteps, int trt, double tau, double tau_anti,
                      const double* force, double* f, double* ftmp, double* rho, double* vel,
                      int nthreads);

/* twophase step (src/twophase/main_TWOPHASE.cpp:238-392) with mass source 0.
 * f, ftmp: LbField(2, N), returned as for oracle_single_run; rho: ScalarField(2, N) holding the fixed solid
 * boundary densities on entry; cg: ScalarField(1, N), zero on entry;
 * force: in/out body force (x is overwritten by the flux controller when
 * flux_control != 0, target mom_x); force_log (may be NULL) receives the
 * body force x used in each step. */
int oracle_twophase_run(const oracle_grid* g, int nsteps, double tau0, double tau1, double sigma,
                        double beta, int flux_control, double mom_x, double* force,
                        double* f, double* ftmp, double* rho, double* vel, double* cg,
                        double* force_log, int nthreads);

/* std_one_phase step (src/std_one_phase/main.cpp:470-575), D3Q19: BGK with the
 * body force times the per-node force attribute, the interior-domain mass
 * sources (calcDeltaOmegaQ) and the solid-fluid, pressure-fluid and
 * fluid-fluid link boundaries of the node tags (main.cpp:24-203).
 * tags, labels, force_on: the nodetags, interior_domains and force attributes,
 * [n_nodes], entry 0 unused (node 0's tag is -1, as Nodes initialises it).
 * rho_w: the pressure-boundary density (the reference passes 1.0).
 * f, ftmp, the return value, rho and vel as for oracle_single_run; flux (may
 * be NULL): the write step's q1, q2 (main.cpp:548-562) after the last step.
 * Returns -20 if an interior domain has no source node (the reference exits). */
int oracle_links_run(const oracle_grid* g, int nsteps, double tau, const double* force, const int32_t* tags,
                     const int32_t* labels, const int32_t* force_on, double rho_w, double* f, double* ftmp,
                     double* rho, double* vel, double* flux, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
