// Host-side launchers of the bclbm kernels (one per kernel family).  Each
// dispatches the run-time lattice / precision / variant choice to a template
// instance and enqueues it on the given stream.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "bclbm_kernels.cuh"

namespace bclbm {

// storage formats: the public precisions, and kFX, the int64 fixed-point storage of
// the default BCLBM_F64 step (not a public precision)
enum Precision { kF64 = 0, kF32 = 1, kF16 = 2, kBF16 = 3, kFX = 4 };

inline int grid_for(int n) { return (n + kBlock - 1) / kBlock; }

// process-wide count of kernel launches issued by the library
std::atomic<int64_t>& launch_counter();

// bclbm_exact.cu (-fmad=false)
cudaError_t launch_single_exact(int Q, bool trt, bool local, const StepArgs& a, cudaStream_t s);
// sums: PASS 1 writes the per-block flux / mass sums (3 per block)
cudaError_t launch_rk_f64(int Q, bool local, bool sums, const StepArgs& a, cudaStream_t s, bool density);

// bclbm_kernels.cu
// pull_map: the tensor map of the handle's pull table (encode_table_map), which
// the native-FP64 steps after the first stage through shared memory; NULL: the
// unstaged kernel
cudaError_t launch_single_fast(int Q, int precision, bool trt, bool local, const StepArgs& a,
                               const CUtensorMap* pull_map, cudaStream_t s);
cudaError_t launch_single_fixed(int Q, bool trt, bool local, const StepArgs& a, cudaStream_t s);
// the tensor map of a [rows][pad] int32 table read in boxes of 32 slots x rows
// (pad a multiple of 64, the table 16-byte aligned)
cudaError_t encode_table_map(const int32_t* table, int pad, int rows, CUtensorMap* out);
cudaError_t launch_rk_shift(int Q, int precision, bool local, bool sums, const StepArgs& a, cudaStream_t s,
                            bool density);
// one pass per step of the shifted two-phase formats (BCLBM_FLAG_LAGGED_COLOUR)
cudaError_t launch_rk_fused(int Q, int precision, bool sums, const StepArgs& a, cudaStream_t s);
cudaError_t launch_flux_force(const double* sum, double inv_n, double mom_x, DevParams* params, cudaStream_t s);
// PASS 2 of the FP64 two-phase step with FMA contraction (BCLBM_FLAG_FP64_FMA)
cudaError_t launch_rk_collide_f64_fma(int Q, bool local, const StepArgs& a, cudaStream_t s);
// the default FP64 two-phase step on the int64 fixed-point state: PASS 1 (density) or PASS 2
cudaError_t launch_rk_fx(int Q, bool local, bool sums, const StepArgs& a, cudaStream_t s, bool density);
cudaError_t launch_rk_fix(const double* sum, double n, double rho_ref, double mom_x, bool flux, int fix,
                          DevParams* params, cudaStream_t s);
cudaError_t launch_gather(int Q, int precision, int nfields, bool local, const StepArgs& a, const int32_t* slot_bulk,
                          double* out, cudaStream_t s);
cudaError_t launch_moments(int Q, int precision, int nfields, bool local, const StepArgs& a, cudaStream_t s);
cudaError_t launch_reduce_final(int nv, const double* partials, int nblocks, double* out, bool max_last,
                                cudaStream_t s);

}  // namespace bclbm
