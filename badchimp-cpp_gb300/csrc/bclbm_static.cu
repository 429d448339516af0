// bclbm_moments_static: FP64 moment sums over a population array the caller
// already holds on the device, for callers that cannot allocate device memory.
//
// Why it exists: bclbm_reduce works on a handle, and creating a handle
// allocates (populations, neighbour table, reduction partials).  Some callers
// cannot allocate at all: a host application whose device memory is owned by
// its own allocator or pool (a stray cudaMalloc would break its accounting or
// its HBM admission budget), or a latency-critical loop where cudaMalloc /
// cudaFree, which may synchronise the whole device, cannot be afforded.  This
// entry point takes device input and output buffers from the caller and keeps
// its only scratch - the per-block partial sums - in a fixed file-scope device
// array, so a call allocates nothing.
//
// Limits and sharing:
//   * at most BCLBM_STATIC_MAX_SLOTS slots (32768 blocks of 256 threads); the
//     scratch is 32768 x 6 doubles = 1.5 MiB, held by every GPU that loads the
//     library until the process exits;
//   * every call on a device uses the same scratch.  A call writes every
//     partial it later reads, so nothing has to start at zero, but calls whose
//     kernels overlap on the GPU (different streams, no ordering between them)
//     race on the scratch and give wrong sums; order them on one stream.
//   * the first call in a CUDA context (the device's primary context, as a
//     rule) looks up the device address of the scratch (cudaGetSymbolAddress)
//     with that context current, and keeps it for that context; make that first
//     call before any stream capture is started on the device.  A device reset
//     (cudaDeviceReset) ends the context: the next call runs in a new one and
//     looks the address up again.
#include <cuda.h>  // CUcontext and the driver entry points' signatures (no libcuda link)
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "bclbm.h"
#include "bclbm_launch.h"

namespace {

constexpr int kStaticMaxBlocks = BCLBM_STATIC_MAX_SLOTS / bclbm::kBlock;
constexpr int kStaticNV = 6;
static_assert(BCLBM_STATIC_MAX_SLOTS % bclbm::kBlock == 0, "slot maximum must be a whole number of blocks");

// The scratch.  In host code this name is only a stand-in for the device array;
// host code must use the address from cudaGetSymbolAddress, never the name.
static __device__ __align__(256) double g_moment_partials[kStaticMaxBlocks * kStaticNV];

// Scratch addresses already looked up, keyed by the unique id of the CUDA
// context they belong to (cuCtxGetId): a reset device, or another context made
// current by the caller, has another id and gets a lookup of its own.
constexpr int kMaxContexts = 64;
std::mutex g_setup_mutex;
struct ScratchEntry {
    unsigned long long ctx_id;
    double* ptr;
};
ScratchEntry g_scratch[kMaxContexts];
int g_n_scratch = 0;

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// The driver's cuCtxGetCurrent / cuCtxGetId through the runtime (the library links
// the runtime only).  Called with g_setup_mutex held.
bool resolve_driver_entry_points() {
    if (g_ctx_get_current && g_ctx_get_id) return true;
    void* a = nullptr;
    void* b = nullptr;
    cudaDriverEntryPointQueryResult qa, qb;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &a, 12000, cudaEnableDefault, &qa) != cudaSuccess ||
        qa != cudaDriverEntryPointSuccess || !a)
        return false;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &b, 12000, cudaEnableDefault, &qb) != cudaSuccess ||
        qb != cudaDriverEntryPointSuccess || !b)
        return false;
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(a);
    g_ctx_get_id = reinterpret_cast<CtxGetIdFn>(b);
    return true;
}

// Id of the context current on this thread, or 0 when none is (yet).
unsigned long long current_context_id() {
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_get_current(&ctx) != CUDA_SUCCESS || !ctx) return 0;
    if (g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch in the current context (looked up once per context).
int scratch_for_current_context(double** out) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return BCLBM_ERR_NOCUDA;
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!resolve_driver_entry_points()) {
        std::fprintf(stderr, "bclbm_moments_static: cuCtxGetCurrent / cuCtxGetId not available from the driver\n");
        return BCLBM_ERR_CUDA;
    }
    unsigned long long id = current_context_id();
    if (id != 0) {
        for (int k = 0; k < g_n_scratch; ++k)
            if (g_scratch[k].ctx_id == id) {
                *out = g_scratch[k].ptr;
                return BCLBM_OK;
            }
    }
    // first call in this context: the lookup also makes the device's primary
    // context current when no context was
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_moment_partials);
    if (e != cudaSuccess || !p) {
        std::fprintf(stderr, "bclbm_moments_static: cudaGetSymbolAddress failed on device %d: %s\n", dev,
                     cudaGetErrorString(e));
        return BCLBM_ERR_CUDA;
    }
    if (id == 0) id = current_context_id();
    if (id != 0) {
        if (g_n_scratch < kMaxContexts) {
            g_scratch[g_n_scratch++] = {id, static_cast<double*>(p)};
        } else {  // table full (contexts come and go): reuse the oldest entry
            for (int k = 1; k < kMaxContexts; ++k) g_scratch[k - 1] = g_scratch[k];
            g_scratch[kMaxContexts - 1] = {id, static_cast<double*>(p)};
        }
    }
    *out = static_cast<double*>(p);
    return BCLBM_OK;
}

// The caller checked that no earlier error was pending, so an error here is these
// launches' own.
template <int Q, class S>
cudaError_t launch(int nfields, const bclbm::StepArgs& a, int nblocks, double* out, cudaStream_t s) {
    using namespace bclbm;
    if (nfields == 1) k_moments<Q, S, 1, true><<<nblocks, kBlock, 0, s>>>(a);
    else k_moments<Q, S, 2, true><<<nblocks, kBlock, 0, s>>>(a);
    launch_counter()++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_reduce_final<kStaticNV><<<1, kFinalThreads, 0, s>>>(a.partials, nblocks, out, 1);
    launch_counter()++;
    return cudaGetLastError();
}

template <int Q>
cudaError_t launch_q(int precision, int nfields, const bclbm::StepArgs& a, int nblocks, double* out, cudaStream_t s) {
    switch (precision) {
        case BCLBM_F64: return launch<Q, double>(nfields, a, nblocks, out, s);
        case BCLBM_F32: return launch<Q, float>(nfields, a, nblocks, out, s);
        case BCLBM_F16: return launch<Q, __half>(nfields, a, nblocks, out, s);
        case BCLBM_BF16: return launch<Q, __nv_bfloat16>(nfields, a, nblocks, out, s);
    }
    return cudaErrorInvalidValue;
}

}  // namespace

extern "C" int bclbm_moments_static(int32_t lattice_q, int32_t precision, int32_t nfields, int32_t n_slots,
                                    int32_t slot_stride, const void* d_pops, double rho_ref, double store_scale,
                                    double* d_out, void* stream) {
    if ((lattice_q != 9 && lattice_q != 19) || precision < BCLBM_F64 || precision > BCLBM_BF16 ||
        (nfields != 1 && nfields != 2) || n_slots < 1 || slot_stride < n_slots || !d_pops || !d_out) {
        std::fprintf(stderr, "bclbm_moments_static: invalid arguments\n");
        return BCLBM_ERR_INVALID;
    }
    if (n_slots > BCLBM_STATIC_MAX_SLOTS) {
        std::fprintf(stderr,
                     "bclbm_moments_static: n_slots = %d exceeds the maximum of %d slots (fixed scratch of %d "
                     "blocks); use bclbm_reduce on a handle for larger lattices\n",
                     n_slots, BCLBM_STATIC_MAX_SLOTS, kStaticMaxBlocks);
        return BCLBM_ERR_INVALID;
    }
    double* scratch = nullptr;
    const int rc = scratch_for_current_context(&scratch);
    if (rc != BCLBM_OK) return rc;
    // an error left by the caller's earlier work is reported as it is and not cleared
    const cudaError_t pending = cudaPeekAtLastError();
    if (pending != cudaSuccess) {
        std::fprintf(stderr, "bclbm_moments_static: an earlier CUDA error is pending (%s); nothing launched\n",
                     cudaGetErrorString(pending));
        return BCLBM_ERR_CUDA;
    }
    bclbm::StepArgs a;
    std::memset(&a, 0, sizeof(a));
    a.L.nf = n_slots;
    a.L.nf_pad = slot_stride;
    a.src = d_pops;
    a.rho_ref = rho_ref > 0 ? rho_ref : 1.0;
    const double scale = store_scale > 0 ? store_scale : (precision == BCLBM_F16 ? 4096.0 : 1.0);
    a.scale = scale;
    a.inv_scale = 1.0 / scale;
    a.f_rho_ref = static_cast<float>(a.rho_ref);  // FP32 copies read by the shifted-format path
    a.f_scale = static_cast<float>(a.scale);
    a.f_inv_scale = static_cast<float>(a.inv_scale);
    a.partials = scratch;
    const int nblocks = bclbm::grid_for(n_slots);
    const cudaStream_t s = static_cast<cudaStream_t>(stream);
    const cudaError_t e = lattice_q == 9 ? launch_q<9>(precision, nfields, a, nblocks, d_out, s)
                                         : launch_q<19>(precision, nfields, a, nblocks, d_out, s);
    if (e != cudaSuccess) {
        std::fprintf(stderr, "bclbm_moments_static: launch failed: %s\n", cudaGetErrorString(e));
        return BCLBM_ERR_CUDA;
    }
    return BCLBM_OK;
}
