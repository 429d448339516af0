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

#ifdef __cplusplus
}
#endif
#endif
