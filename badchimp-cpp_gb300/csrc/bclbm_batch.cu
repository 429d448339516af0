// Multi-instance batch: many lattice instances resident in HBM, stepped together
// by one persistent kernel over a concatenated work list, in blocks of steps
// replayed from a captured CUDA graph.
//
// Instances are ordinary handles (bclbm_create builds and uploads them); the
// batch keeps, in device memory,
//   inst[slot]  the kernel arguments of each admitted instance and the global
//               step at which it was admitted;
//   work[w]     (slot, first fluid slot) of every 256-node block of every
//               admitted instance, instances contiguous;
//   n_work, step  the work-list length and the global step counter;
//   ctr         the item counter, from which the persistent kernel's blocks
//               (a fixed grid, one wave) take items in list order, and a count
//               of finished blocks: the last block of a step advances step and
//               rewinds both, so one launch is one step.
// The persistent kernel reads all of them at run time, so its launch parameters
// never change and the graph captured once stays valid while instances are
// admitted and retired between replays.  An instance's ping-pong parity follows
// from (step - admitted_step), so instances that joined at different times
// advance together.  Admission takes the instance's first step (the one that
// reads the initial populations in place) with the single-instance kernel, so
// the batch kernel only has the pull form.
//
// Per-instance results are independent of the other instances: each node's
// arithmetic is the single-instance kernel's, and the FP64 reductions sum the
// same 256-node blocks in the same order as bclbm_reduce does.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <type_traits>
#include <vector>

#include "bclbm.h"
#include "bclbm_internal.h"
#include "bclbm_trace.h"
#include "bclbm_launch.h"

using namespace bclbm;

namespace {

struct BatchInst {
    StepArgs args;         // src, dst and macro outputs are set per step
    void* pops[2];
    long long start_step;  // global step at admission
    double force[3];
};

template <int Q, class S, int MODE, bool TRT>
__device__ __forceinline__ void batch_node(const StepArgs& a, int i) {
    if constexpr (MODE == 2) fixed_node<Q, TRT, false>(a, i);
    else single_node<Q, S, MODE, TRT, false>(a, i);
}

// Loads the arguments of instance `slot` into shared memory and sets the
// parity-dependent pointers.  Called by every thread of the block.
__device__ __forceinline__ void load_inst(const BatchInst* __restrict__ inst, int slot, long long step, StepArgs& a) {
    __syncthreads();
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&inst[slot].args);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&a);
    for (int k = threadIdx.x; k < static_cast<int>(sizeof(StepArgs) / 4); k += blockDim.x) dst[k] = src[k];
    __syncthreads();
    if (threadIdx.x == 0) {
        const long long age = step - inst[slot].start_step;
        const int par = static_cast<int>(age & 1);
        a.src = inst[slot].pops[par];
        a.dst = inst[slot].pops[par ^ 1];
        a.rho_out = nullptr;
        a.vel_out = nullptr;
    }
    __syncthreads();
}

// resident blocks per SM asked of the register allocator: the kernel arguments
// live in shared memory, and without a bound the allocator keeps them all in
// registers across the item loop (FP16/FP32: 85 instead of the ~62 of the
// single-instance kernel, one block per SM fewer); 5 blocks per SM squeeze it to
// 48 registers with spills (24-request serving sample, FP32: 27.3 -> 22.1 GLUPS)
#ifndef BCLBM_BATCH_SHIFT_MINB
#define BCLBM_BATCH_SHIFT_MINB 4
#endif
template <class S, int MODE>
constexpr int batch_min_blocks() {
    return MODE == 2 ? 3 : (std::is_same<S, double>::value ? 2 : BCLBM_BATCH_SHIFT_MINB);
}

template <int Q, class S, int MODE, bool TRT>
__global__ void __launch_bounds__(kBlock, batch_min_blocks<S, MODE>()) k_batch_step(const BatchInst* __restrict__ inst,
                                                       const int2* __restrict__ work, const int* n_work,
                                                       long long* step, int* ctr) {
    __shared__ __align__(16) unsigned char smem[sizeof(StepArgs)];
    __shared__ int s_item;
    __shared__ int s_last;
    int* next_item = ctr;  // ctr[0]: next item; ctr[1]: blocks finished
    StepArgs& a = *reinterpret_cast<StepArgs*>(smem);
    const long long st = *step;
    const int nw = *n_work;
    // Items are taken from a counter in list order, as the hardware hands out the
    // blocks of an ordinary launch: the items in flight stay a compact window of
    // the node list, whose upstream neighbours are still in L2 (a static
    // grid-stride split lets the blocks drift apart: 20% slower on 256^3).
    int cur = -1;
    // Items are taken two at a time (one counter operation and one pair of barriers
    // per 512 nodes: +3-6% over single items, less with four).
    constexpr int kTake = 2;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(next_item, 1);
        __syncthreads();
        const int w0 = kTake * s_item;
        if (w0 >= nw) break;
        const int wend = min(w0 + kTake, nw);
        for (int w = w0; w < wend; ++w) {
            const int2 wk = work[w];
            if (wk.x != cur) {
                load_inst(inst, wk.x, st, a);
                cur = wk.x;
            }
            const int i = wk.y + threadIdx.x;
            if (i < a.L.nf) batch_node<Q, S, MODE, TRT>(a, i);
        }
        __syncthreads();  // s_item is rewritten at the next take
    }
    // the last block to finish advances the step and rewinds the counters for the
    // next launch; every block has read *step before it counts itself finished
    if (threadIdx.x == 0) {
        __threadfence();
        s_last = atomicAdd(&ctr[1], 1) == static_cast<int>(gridDim.x) - 1;
    }
    __syncthreads();
    if (s_last && threadIdx.x == 0) {
        *step = st + 1;
        ctr[0] = 0;
        ctr[1] = 0;
        __threadfence();
    }
}

template <int Q, class S>
__global__ void __launch_bounds__(kBlock) k_batch_moments(const BatchInst* __restrict__ inst,
                                                          const int2* __restrict__ work, const int* n_work,
                                                          const long long* step, double* partials) {
    __shared__ __align__(16) unsigned char smem[sizeof(StepArgs)];
    StepArgs& a = *reinterpret_cast<StepArgs*>(smem);
    const long long st = *step;
    const int nw = *n_work;
    int cur = -1;
    for (int w = blockIdx.x; w < nw; w += gridDim.x) {
        const int2 wk = work[w];
        if (wk.x != cur) {
            load_inst(inst, wk.x, st, a);
            cur = wk.x;
        }
        double vals[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        const int i = wk.y + threadIdx.x;
        // the state of an instance is in pops[age & 1], which load_inst put in src
        if (i < a.L.nf) moments_node<Q, S, 1, false>(a, i, vals);
        block_reduce_store<6>(vals, partials, true, w);
        __syncthreads();
    }
}

// one block per requested instance: its work items' partials, summed exactly as
// bclbm_reduce sums a handle's block partials (final_sum)
__global__ void __launch_bounds__(kFinalThreads) k_batch_final(const double* __restrict__ partials,
                                                              const int* __restrict__ first,
                                                              const int* __restrict__ count, double* out) {
    const int j = blockIdx.x;
    final_sum<6>(partials + static_cast<size_t>(first[j]) * 6, count[j], out + static_cast<size_t>(j) * 6, true);
}

using StepKernel = void (*)(const BatchInst*, const int2*, const int*, long long*, int*);
using MomKernel = void (*)(const BatchInst*, const int2*, const int*, const long long*, double*);

template <int Q>
StepKernel pick_step(int precision, int mode, bool trt) {
    if (mode == 2) return trt ? k_batch_step<Q, double, 2, true> : k_batch_step<Q, double, 2, false>;
    switch (precision) {
        case BCLBM_F64: return trt ? k_batch_step<Q, double, 1, true> : k_batch_step<Q, double, 1, false>;
        case BCLBM_F32: return trt ? k_batch_step<Q, float, 1, true> : k_batch_step<Q, float, 1, false>;
        case BCLBM_F16: return trt ? k_batch_step<Q, __half, 1, true> : k_batch_step<Q, __half, 1, false>;
        case BCLBM_BF16:
            return trt ? k_batch_step<Q, __nv_bfloat16, 1, true> : k_batch_step<Q, __nv_bfloat16, 1, false>;
    }
    return nullptr;
}

template <int Q>
MomKernel pick_mom(int precision) {
    switch (precision) {
        case BCLBM_F64: return k_batch_moments<Q, double>;
        case BCLBM_F32: return k_batch_moments<Q, float>;
        case BCLBM_F16: return k_batch_moments<Q, __half>;
        case BCLBM_BF16: return k_batch_moments<Q, __nv_bfloat16>;
    }
    return nullptr;
}

}  // namespace

struct bclbm_batch {
    int q = 0, collision = 0, precision = 0, mode = 1;
    uint32_t flags = 0;
    int max_inst = 0, max_work = 0, graph_steps = 0, grid = 0;
    size_t budget = 0, used = 0;
    std::vector<bclbm_handle*> handle;  // per slot, nullptr = free
    std::vector<size_t> bytes;          // per slot footprint
    std::vector<long long> start;       // per slot admission step
    std::vector<int> wfirst, wcount;    // per slot work range
    int n_work = 0;
    bool dirty = false;
    long long host_step = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    BatchInst* d_inst = nullptr;
    int2* d_work = nullptr;
    int* d_nwork = nullptr;
    long long* d_step = nullptr;
    int* d_ctr = nullptr;  // step kernel counters: next item, blocks finished
    double* d_partials = nullptr;
    int* d_first = nullptr;
    int* d_count = nullptr;
    double* d_out = nullptr;
    StepKernel step_kernel = nullptr;
    MomKernel mom_kernel = nullptr;
    cudaGraphExec_t graph = nullptr;
    std::string last_error;
};

namespace {

int bfail(bclbm_batch* b, int code, const std::string& msg) {
    if (b) b->last_error = msg;
    return code;
}

#define BTRY(b, expr)                                                                                 \
    do {                                                                                              \
        cudaError_t e_ = (expr);                                                                      \
        if (e_ != cudaSuccess)                                                                        \
            return bfail((b), e_ == cudaErrorMemoryAllocation ? BCLBM_ERR_NOMEM : BCLBM_ERR_CUDA,       \
                         std::string(#expr) + ": " + cudaGetErrorString(e_));                           \
    } while (0)

void batch_free(bclbm_batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    cudaFree(b->d_inst);
    cudaFree(b->d_work);
    cudaFree(b->d_nwork);
    cudaFree(b->d_step);
    cudaFree(b->d_ctr);
    cudaFree(b->d_partials);
    cudaFree(b->d_first);
    cudaFree(b->d_count);
    cudaFree(b->d_out);
    if (b->stream) cudaStreamDestroy(b->stream);
}

// Rebuilds the work list (instances in slot order, 256-node blocks) and uploads it.
int upload_work(bclbm_batch* b) {
    std::vector<int2> work;
    for (int s = 0; s < b->max_inst; ++s) {
        b->wfirst[s] = static_cast<int>(work.size());
        b->wcount[s] = 0;
        if (!b->handle[s]) continue;
        const int nf = b->handle[s]->nf;
        for (int base = 0; base < nf; base += kBlock) work.push_back(make_int2(s, base));
        b->wcount[s] = static_cast<int>(work.size()) - b->wfirst[s];
    }
    if (static_cast<int>(work.size()) > b->max_work) {
        // grow the work list and its partials; the captured graph holds the old
        // pointers, so it is dropped and captured again at the next replay
        int cap = std::max(b->max_work, 1024);
        while (cap < static_cast<int>(work.size())) cap *= 2;
        int2* nw = nullptr;
        double* np = nullptr;
        if (cudaMalloc(&nw, sizeof(int2) * cap) != cudaSuccess ||
            cudaMalloc(&np, sizeof(double) * 6 * static_cast<size_t>(cap)) != cudaSuccess) {
            cudaFree(nw);
            return bfail(b, BCLBM_ERR_NOMEM, "work list allocation failed");
        }
        cudaFree(b->d_work);
        cudaFree(b->d_partials);
        b->d_work = nw;
        b->d_partials = np;
        b->max_work = cap;
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
    }
    b->n_work = static_cast<int>(work.size());
    if (!work.empty())
        BTRY(b, cudaMemcpyAsync(b->d_work, work.data(), work.size() * sizeof(int2), cudaMemcpyHostToDevice, b->stream));
    BTRY(b, cudaMemcpyAsync(b->d_nwork, &b->n_work, sizeof(int), cudaMemcpyHostToDevice, b->stream));
    BTRY(b, cudaStreamSynchronize(b->stream));
    b->dirty = false;
    return BCLBM_OK;
}

int launch_steps_direct(bclbm_batch* b, int n) {
    for (int k = 0; k < n; ++k) {
        b->step_kernel<<<b->grid, kBlock, 0, b->stream>>>(b->d_inst, b->d_work, b->d_nwork, b->d_step, b->d_ctr);
        launch_counter() += 1;
    }
    BTRY(b, cudaGetLastError());
    return BCLBM_OK;
}

int ensure_graph(bclbm_batch* b) {
    if (b->graph || b->graph_steps <= 0) return BCLBM_OK;
    cudaGraph_t g = nullptr;
    BTRY(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    for (int k = 0; k < b->graph_steps; ++k) {
        b->step_kernel<<<b->grid, kBlock, 0, b->stream>>>(b->d_inst, b->d_work, b->d_nwork, b->d_step, b->d_ctr);
    }
    const cudaError_t ec = cudaStreamEndCapture(b->stream, &g);
    if (ec != cudaSuccess) return bfail(b, BCLBM_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ec));
    const cudaError_t ei = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        b->graph = nullptr;
        return bfail(b, BCLBM_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ei));
    }
    return BCLBM_OK;
}

}  // namespace

extern "C" {

int bclbm_batch_create(int32_t lattice_q, int32_t collision, int32_t precision, uint32_t flags, int32_t max_instances,
                       size_t hbm_budget, int32_t steps_per_graph, bclbm_batch** out) {
    if (!out) return BCLBM_ERR_INVALID;
    *out = nullptr;
    if ((lattice_q != 9 && lattice_q != 19) || (collision != BCLBM_BGK && collision != BCLBM_TRT) ||
        precision < BCLBM_F64 || precision > BCLBM_BF16 || max_instances < 1 || hbm_budget == 0 || steps_per_graph < 0)
        return BCLBM_ERR_INVALID;
    // the reference-order kernel lives in the -fmad=false unit; batches use the fixed-point
    // FP64 step (bit-reproducible) or the FMA / shifted-storage steps
    if (flags & BCLBM_FLAG_EXACT) return BCLBM_ERR_UNSUPPORTED;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return BCLBM_ERR_NOCUDA;
    bclbm_batch* b = new (std::nothrow) bclbm_batch();
    if (!b) return BCLBM_ERR_NOMEM;
    b->q = lattice_q;
    b->collision = collision;
    b->precision = precision;
    b->flags = flags;
    b->mode = (precision == BCLBM_F64 && !(flags & BCLBM_FLAG_FP64_FMA)) ? 2 : 1;
    b->max_inst = max_instances;
    b->budget = hbm_budget;
    b->graph_steps = steps_per_graph;
    b->max_work = 1024;  // grows with the admitted instances
    b->handle.assign(max_instances, nullptr);
    b->bytes.assign(max_instances, 0);
    b->start.assign(max_instances, 0);
    b->wfirst.assign(max_instances, 0);
    b->wcount.assign(max_instances, 0);
    cudaGetDevice(&b->device);
    const bool trt = collision == BCLBM_TRT;
    b->step_kernel = lattice_q == 9 ? pick_step<9>(precision, b->mode, trt) : pick_step<19>(precision, b->mode, trt);
    // the fixed-point step keeps int64 storage (Store<int64_t>)
    b->mom_kernel = b->mode == 2 ? (lattice_q == 9 ? k_batch_moments<9, int64_t> : k_batch_moments<19, int64_t>)
                                 : (lattice_q == 9 ? pick_mom<9>(precision) : pick_mom<19>(precision));
    auto cleanup = [&](int code) {
        batch_free(b);
        delete b;
        return code;
    };
    int nsm = 0, per_sm = 0;
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, b->device) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, b->step_kernel, kBlock, 0) != cudaSuccess)
        return cleanup(BCLBM_ERR_CUDA);
    b->grid = std::max(1, nsm * std::max(1, per_sm));
    if (cudaMalloc(&b->d_inst, sizeof(BatchInst) * max_instances) != cudaSuccess ||
        cudaMalloc(&b->d_work, sizeof(int2) * b->max_work) != cudaSuccess ||
        cudaMalloc(&b->d_nwork, sizeof(int)) != cudaSuccess || cudaMalloc(&b->d_step, sizeof(long long)) != cudaSuccess ||
        cudaMalloc(&b->d_ctr, 2 * sizeof(int)) != cudaSuccess ||
        cudaMalloc(&b->d_partials, sizeof(double) * 6 * static_cast<size_t>(b->max_work)) != cudaSuccess ||
        cudaMalloc(&b->d_first, sizeof(int) * max_instances) != cudaSuccess ||
        cudaMalloc(&b->d_count, sizeof(int) * max_instances) != cudaSuccess ||
        cudaMalloc(&b->d_out, sizeof(double) * 6 * max_instances) != cudaSuccess)
        return cleanup(BCLBM_ERR_NOMEM);
    const int zero = 0;
    const long long zstep = 0;
    if (cudaMemcpyAsync(b->d_nwork, &zero, sizeof(int), cudaMemcpyHostToDevice, b->stream) != cudaSuccess ||
        cudaMemsetAsync(b->d_ctr, 0, 2 * sizeof(int), b->stream) != cudaSuccess ||
        cudaMemcpyAsync(b->d_step, &zstep, sizeof(long long), cudaMemcpyHostToDevice, b->stream) != cudaSuccess ||
        cudaStreamSynchronize(b->stream) != cudaSuccess)
        return cleanup(BCLBM_ERR_CUDA);
    *out = b;
    return BCLBM_OK;
}

int bclbm_batch_admit(bclbm_batch* b, const bclbm_desc* desc, int32_t* id) {
    return bclbm_batch_admit_steps(b, desc, 1, id);
}

int bclbm_batch_attach(bclbm_batch* b, bclbm_handle* h, int32_t* id) {
    if (!b || !h || !id) return BCLBM_ERR_INVALID;
    *id = -1;
    if (h->q != b->q || h->collision != b->collision || h->precision != b->precision || h->exact ||
        h->fma64 != ((b->flags & BCLBM_FLAG_FP64_FMA) != 0))
        return bfail(b, BCLBM_ERR_INVALID, "handle does not match the batch's lattice, collision or precision");
    if (h->steps_done < 1 || !h->state_post)
        return bfail(b, BCLBM_ERR_INVALID, "attach needs a handle that has taken at least one step");
    for (int s = 0; s < b->max_inst; ++s)
        if (b->handle[s] == h) return bfail(b, BCLBM_ERR_INVALID, "handle already attached");
    const size_t need = h->footprint;
    int slot = -1;
    for (int s = 0; s < b->max_inst; ++s)
        if (!b->handle[s]) {
            slot = s;
            break;
        }
    if (slot < 0 || b->used + need > b->budget) return bfail(b, BCLBM_ERR_BUDGET, "no free slot or HBM budget");
    BTRY(b, cudaSetDevice(b->device));
    BTRY(b, cudaStreamSynchronize(h->stream));
    BTRY(b, cudaStreamSynchronize(b->stream));
    BatchInst bi;
    std::memset(&bi, 0, sizeof(bi));
    bi.args = handle_args(h);
    bi.pops[0] = h->pops[0];
    bi.pops[1] = h->pops[1];
    // the state is in pops[steps_done & 1] (== h->cur); start_step keeps that parity
    bi.start_step = b->host_step - h->steps_done;
    for (int k = 0; k < 3; ++k) bi.force[k] = h->force[k];
    BTRY(b, cudaMemcpyAsync(b->d_inst + slot, &bi, sizeof(bi), cudaMemcpyHostToDevice, b->stream));
    b->handle[slot] = h;
    b->bytes[slot] = need;
    b->start[slot] = bi.start_step;
    b->used += need;
    const int rc = upload_work(b);
    if (rc) return rc;
    *id = slot;
    return BCLBM_OK;
}

int bclbm_batch_admit_steps(bclbm_batch* b, const bclbm_desc* desc, int32_t first_steps, int32_t* id) {
    BCLBM_TRACE("bclbm_batch_admit");
    if (!b || !desc || !id || first_steps < 1) return BCLBM_ERR_INVALID;
    *id = -1;
    if (desc->lattice_q != b->q || desc->collision != b->collision || desc->precision != b->precision ||
        (desc->flags & (BCLBM_FLAG_EXACT | BCLBM_FLAG_FP64_FMA)) != (b->flags & (BCLBM_FLAG_EXACT | BCLBM_FLAG_FP64_FMA)))
        return bfail(b, BCLBM_ERR_INVALID, "descriptor does not match the batch's lattice, collision or precision");
    size_t need = 0;
    int rc = bclbm_footprint(desc, &need);
    if (rc) return rc;
    int free_slots = 0;
    for (auto* x : b->handle) free_slots += x == nullptr;
    if (free_slots == 0 || b->used + need > b->budget) return bfail(b, BCLBM_ERR_BUDGET, "no free slot or HBM budget");
    BTRY(b, cudaSetDevice(b->device));
    bclbm_handle* h = nullptr;
    rc = bclbm_create(desc, &h);
    if (rc) return bfail(b, rc, std::string("instance creation: ") + bclbm_error(rc));
    rc = bclbm_step(h, first_steps);
    if (rc) {
        b->last_error = std::string("first steps: ") + bclbm_last_error(h);
        bclbm_destroy(h);
        return rc;
    }
    rc = bclbm_batch_attach(b, h, id);
    if (rc) bclbm_destroy(h);
    return rc;
}

int bclbm_batch_retire(bclbm_batch* b, int32_t id) {
    if (!b || id < 0 || id >= b->max_inst || !b->handle[id]) return BCLBM_ERR_INVALID;
    BTRY(b, cudaSetDevice(b->device));
    BTRY(b, cudaStreamSynchronize(b->stream));
    bclbm_destroy(b->handle[id]);
    b->handle[id] = nullptr;
    b->used -= b->bytes[id];
    b->bytes[id] = 0;
    return upload_work(b);
}

int bclbm_batch_step(bclbm_batch* b, int32_t nsteps) {
    BCLBM_TRACE("bclbm_batch_step");
    if (!b || nsteps < 0) return BCLBM_ERR_INVALID;
    BTRY(b, cudaSetDevice(b->device));
    int rc = BCLBM_OK;
    int left = nsteps;
    if (b->graph_steps > 0 && left >= b->graph_steps) {
        rc = ensure_graph(b);
        if (rc) return rc;
        while (left >= b->graph_steps) {
            BTRY(b, cudaGraphLaunch(b->graph, b->stream));
            launch_counter() += b->graph_steps;
            left -= b->graph_steps;
        }
    }
    rc = launch_steps_direct(b, left);
    if (rc) return rc;
    b->host_step += nsteps;
    return BCLBM_OK;
}

int bclbm_batch_stats(bclbm_batch* b, int32_t n, const int32_t* ids, bclbm_stats* out) {
    BCLBM_TRACE("bclbm_batch_stats");
    if (!b || n < 0 || n > b->max_inst || (n > 0 && (!ids || !out))) return BCLBM_ERR_INVALID;
    if (n == 0) return BCLBM_OK;
    BTRY(b, cudaSetDevice(b->device));
    std::vector<int> first(n), count(n);
    for (int j = 0; j < n; ++j) {
        const int s = ids[j];
        if (s < 0 || s >= b->max_inst || !b->handle[s]) return bfail(b, BCLBM_ERR_INVALID, "unknown instance id");
        first[j] = b->wfirst[s];
        count[j] = b->wcount[s];
    }
    b->mom_kernel<<<b->grid, kBlock, 0, b->stream>>>(b->d_inst, b->d_work, b->d_nwork, b->d_step, b->d_partials);
    launch_counter()++;
    BTRY(b, cudaMemcpyAsync(b->d_first, first.data(), n * sizeof(int), cudaMemcpyHostToDevice, b->stream));
    BTRY(b, cudaMemcpyAsync(b->d_count, count.data(), n * sizeof(int), cudaMemcpyHostToDevice, b->stream));
    k_batch_final<<<n, kFinalThreads, 0, b->stream>>>(b->d_partials, b->d_first, b->d_count, b->d_out);
    launch_counter()++;
    BTRY(b, cudaGetLastError());
    std::vector<double> res(static_cast<size_t>(n) * 6);
    std::vector<DevParams> prm(n);
    BTRY(b, cudaMemcpyAsync(res.data(), b->d_out, res.size() * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    for (int j = 0; j < n; ++j)
        BTRY(b, cudaMemcpyAsync(&prm[j], b->handle[ids[j]]->d_params, sizeof(DevParams), cudaMemcpyDeviceToHost,
                                b->stream));
    BTRY(b, cudaStreamSynchronize(b->stream));
    int rc = BCLBM_OK;
    for (int j = 0; j < n; ++j) {
        const bclbm_handle* h = b->handle[ids[j]];
        const double* r = res.data() + static_cast<size_t>(j) * 6;
        bclbm_stats& st = out[j];
        std::memset(&st, 0, sizeof(st));
        st.mass[0] = r[0];
        st.mass[1] = r[1];
        for (int k = 0; k < 3; ++k) {
            st.flux_fc[k] = r[2 + k];
            st.momentum[k] = r[2 + k] + 0.5 * h->force[k] * static_cast<double>(h->nf);
        }
        st.max_abs_f = r[5];
        st.n_bulk = h->nf;
        st.steps_done = b->host_step - b->start[ids[j]];
        st.nonfinite = std::isfinite(r[5]) && std::isfinite(r[0]) ? 0 : 1;
        if (prm[j].fx_overflow & stage::kFlagWaitTimeout) {
            rc = bfail(b, BCLBM_ERR_CUDA, "a step kernel's bounded wait for a staged table tile ran out");
        } else if (prm[j].fx_overflow) {
            st.nonfinite = 1;
            rc = bfail(b, BCLBM_ERR_NONFINITE, "a node left the fixed-point range (sum |f| < 8, rho > 0.15)");
        } else if (st.nonfinite && rc == BCLBM_OK) {
            rc = bfail(b, BCLBM_ERR_NONFINITE, "NaN or Inf in the populations");
        }
    }
    return rc;
}

int bclbm_batch_download_f(bclbm_batch* b, int32_t id, double* f) {
    if (!b || id < 0 || id >= b->max_inst || !b->handle[id] || !f) return BCLBM_ERR_INVALID;
    BTRY(b, cudaSetDevice(b->device));
    BTRY(b, cudaStreamSynchronize(b->stream));
    bclbm_handle* h = b->handle[id];
    const long long age = b->host_step - b->start[id];
    h->cur = static_cast<int>(age & 1);
    h->state_post = age > 0;
    return bclbm_download_f(h, f);
}

int bclbm_batch_info(bclbm_batch* b, size_t* used_bytes, int32_t* n_active, int64_t* steps) {
    if (!b) return BCLBM_ERR_INVALID;
    int n = 0;
    for (auto* h : b->handle) n += h != nullptr;
    if (used_bytes) *used_bytes = b->used;
    if (n_active) *n_active = n;
    if (steps) *steps = b->host_step;
    return BCLBM_OK;
}

int bclbm_batch_sync(bclbm_batch* b) {
    if (!b) return BCLBM_ERR_INVALID;
    BTRY(b, cudaStreamSynchronize(b->stream));
    return BCLBM_OK;
}

const char* bclbm_batch_last_error(const bclbm_batch* b) { return b ? b->last_error.c_str() : ""; }

void bclbm_batch_destroy(bclbm_batch* b) {
    if (!b) return;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (auto*& h : b->handle)
        if (h) {
            bclbm_destroy(h);
            h = nullptr;
        }
    batch_free(b);
    delete b;
}

}  // extern "C"
