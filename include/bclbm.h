/*
 * bclbm: GB300-native (sm_103a) lattice-Boltzmann time step for BADChIMP.
 *
 * C ABI.  Plain pointers and sizes only; no exceptions cross it, nothing here
 * calls exit().  Every function returns BCLBM_OK (0) or a negative status whose
 * text bclbm_error() gives; bclbm_last_error() adds the detail of the last
 * failure on a handle.
 *
 * The boundary replaces, in the reference's main-file time loops, the per-node
 * collide/propagate loops, LbField::swapData, BndMpi::communicate* (a no-op at
 * one rank) and HalfWayBounceBack::apply:
 *   src/std_case/main.cpp:110-145         one bclbm_step(h, 1) per iteration
 *   src/twophase/main_TWOPHASE.cpp:238-392 one bclbm_step(h, 1) per iteration
 * Output steps (std_case/main.cpp:150-155, main_TWOPHASE.cpp:399-448) call
 * bclbm_download_macros() into the reference's ScalarField/VectorField storage
 * before Output::write().
 *
 * All host arrays passed in or out use the reference's layout and node
 * numbering:
 *   neigh   [N*Q]      Grid::neigList_           (src/lbsolver/LBgrid.h:119, 160, 197)
 *   types   [N]        Nodes::nodeType_          (src/lbsolver/LBnodes.h:107, 156-209)
 *   bulk    [n_bulk]   findBulkNodes()           (src/lbsolver/LBgeometry.h:11-21)
 *   f       [N*nF*Q]   LbField data_             (src/lbsolver/LBfield.h:298-305)
 *   rho     [N*nF]     ScalarField data_         (src/lbsolver/LBfield.h:92-100)
 *   vel     [N*nD]     VectorField data_, 1 field (src/lbsolver/LBfield.h:168-175)
 *   cg      [N]        the twophase colour field cgField (main_TWOPHASE.cpp:144, 245, 283)
 * with N = Grid::size() (node 0 is the ghost node), Q = 9 (D2Q9) or 19 (D3Q19).
 *
 * A handle owns one lattice instance on the current CUDA device and a stream
 * of its own; calls on one handle come from one host thread.  bclbm_step() is
 * asynchronous; downloads and reductions synchronise the handle's stream.
 */
#ifndef BCLBM_H
#define BCLBM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BCLBM_ABI_VERSION 1

/* status codes */
#define BCLBM_OK 0
#define BCLBM_ERR_INVALID (-1)     /* bad argument or descriptor */
#define BCLBM_ERR_TABLE (-2)       /* neighbour table / node types inconsistent */
#define BCLBM_ERR_NOMEM (-3)       /* device or host allocation failed */
#define BCLBM_ERR_CUDA (-4)        /* CUDA runtime error */
#define BCLBM_ERR_UNSUPPORTED (-5) /* combination not built */
#define BCLBM_ERR_NONFINITE (-6)   /* NaN/Inf found by a reduction */
#define BCLBM_ERR_BUDGET (-7)      /* request exceeds the HBM admission budget */
#define BCLBM_ERR_NOCUDA (-8)      /* no CUDA device visible */

/* collision models */
#define BCLBM_BGK 0 /* calcOmegaBGK + calcDeltaOmegaF          (src/lbsolver/LBcollision.h:27-46, 194-213) */
#define BCLBM_TRT 1 /* calcOmegaBGKTRT + calcDeltaOmegaFTRT(phi=1) (LBcollision.h:50-75, 215-236) */
#define BCLBM_RK 2  /* Rothman-Keller two-phase step of src/twophase/main_TWOPHASE.cpp:238-392;
                       BCLBM_F64: both colour sets and the colour field in 64-bit fixed point, every
                       term of the collision a fixed-point product (default; needs |sigma| < 3.5 and
                       |beta| < 4), the reference's rounding with BCLBM_FLAG_EXACT, FP64 with FMA
                       under BCLBM_FLAG_FP64_FMA; BCLBM_F32 / F16 / BF16: shifted storage with FP32
                       arithmetic (one pass per step with BCLBM_FLAG_LAGGED_COLOUR) */
#define BCLBM_LINKS 3 /* the std_one_phase step (src/std_one_phase/main.cpp:470-575, D3Q19):
                         BGK + Guo force times the per-node force attribute, interior-domain mass
                         sources (calcDeltaOmegaQ) and the solid-fluid, pressure (anti-bounce-back)
                         and fluid-fluid link boundaries of the node tags.  BCLBM_F64: FP64 storage
                         with the 64-bit fixed-point collision of the std_case step (default), FP64
                         with FMA under BCLBM_FLAG_FP64_FMA, or the reference's rounding with
                         FLAG_EXACT; BCLBM_F32 / F16 / BF16: shifted storage with FP32 arithmetic on
                         the deviations */

/* population storage on the device */
#define BCLBM_F64 0  /* plain FP64 populations; arithmetic: 64-bit fixed point with 2^-60
                        resolution (finer than an FP64 ulp of any population of a fluid
                        with rho ~ 1; needs sum_q |f_q| < 8 and rho > 0.15 per node,
                        else bclbm_reduce reports BCLBM_ERR_NONFINITE), results rounded
                        to FP64; the single-phase collision needs tau > 0.5 (and
                        tau_anti > 0.5 for TRT).  With
                        BCLBM_FLAG_EXACT: FP64 in the reference's expression order;
                        with BCLBM_FLAG_FP64_FMA: FP64 with FMA (any parameters). */
#define BCLBM_F32 1  /* FP32 shifted deviations (f - w*rho_ref)/w, FP32 arithmetic */
#define BCLBM_F16 2  /* FP16 shifted, scaled deviations, FP32 arithmetic */
#define BCLBM_BF16 3 /* BF16 shifted, scaled deviations, FP32 arithmetic */

/* flags */
#define BCLBM_FLAG_EXACT 1u     /* FP64 only: the reference's expression order, no FMA
                                   contraction: results bit-identical to the reference */
#define BCLBM_FLAG_SFC_ORDER 2u /* reorder fluid nodes along a Morton curve of their
                                   positions (needs pos); downloads keep reference order */
#define BCLBM_FLAG_FP64_FMA 4u  /* BCLBM_F64: native FP64 arithmetic with FMA (single phase:
                                   instead of the fixed point; two-phase: instead of the
                                   reference's rounding order) */
#define BCLBM_FLAG_NO_MASS_FIX 8u /* two-phase shifted storage: switch off the per-step correction
                                     that restores the two conserved totals, sum (f0 + f1) and
                                     sum (f0 - f1), from an FP64 reduction (rounding of the
                                     stored values does not conserve them) */
#define BCLBM_FLAG_LAGGED_COLOUR 16u /* two-phase shifted storage (F32 / F16 / BF16): one pass per
                                        step instead of two.  The colour gradient of step t takes the
                                        neighbours' colours of step t - 1 (the step's own colour and
                                        densities stay current), and the flux controller's force and
                                        the mass correction computed in step t apply from step t + 1.
                                        Not the reference's ordering (main_TWOPHASE.cpp:238-376 forms
                                        every colour before any collision); the first step after
                                        bclbm_create runs both passes. */

typedef struct {
    int32_t lattice_q;        /* 9 or 19 */
    int32_t n_nodes;          /* N = Grid::size() */
    const int32_t* neigh;     /* [N*Q] */
    const int16_t* types;     /* [N] */
    int32_t n_bulk;           /* number of bulk (own-rank fluid) nodes; the steps index the
                                 populations with 32-bit element numbers, so Q times n_bulk
                                 (rounded up to a multiple of 64) must stay below 2^31
                                 (D3Q19: 113 M nodes), else BCLBM_ERR_UNSUPPORTED */
    const int32_t* bulk;      /* [n_bulk], increasing; every listed node has type > 1 */
    const int32_t* pos;       /* [N*nD] Grid positions, needed for BCLBM_FLAG_SFC_ORDER, else NULL */
    int32_t collision;        /* BCLBM_BGK | BCLBM_TRT | BCLBM_RK */
    int32_t precision;        /* BCLBM_F64 | BCLBM_F32 | BCLBM_F16 | BCLBM_BF16 */
    uint32_t flags;
    double tau[2];            /* BGK: tau[0]; TRT: tau[0] symmetric, tau[1] antisymmetric;
                                 RK: the two phase relaxation times (fluid.tau[0], fluid.tau[1]) */
    double force[3];          /* body force (VectorField bodyForce(1,1)); unused components 0 */
    double sigma;             /* RK: surface tension parameter A (fluid.sigma) */
    double beta;              /* RK: recolouring parameter (fluid.beta) */
    int32_t flux_control;     /* RK: 1 = body force x from the flux controller of
                                 main_TWOPHASE.cpp:292-308 every step, target mom_x */
    double mom_x;             /* RK: fluid.momx */
    double rho_ref;           /* shifted storage: reference density of the shift (1.0 if 0) */
    double store_scale;       /* F16/BF16: scale of the stored deviations (default if 0) */
    const double* f_init;     /* [N*nF*Q] initial populations, nF = 2 for RK else 1 */
    const double* rho_init;   /* RK: [N*2] densities; only the solid boundary entries (type 1)
                                 are read (the wettability densities); else NULL */
    /* BCLBM_LINKS: the nodetags, interior_domains and force attributes, [N] each (entry 0
       unused: node 0's tag is -1, as Nodes initialises it; force_on NULL = 1 everywhere),
       and the pressure-boundary density (0: 1.0, the value main.cpp:537 passes) */
    const int32_t* tags;
    const int32_t* labels;
    const int32_t* force_on;
    double rho_w;
} bclbm_desc;

typedef struct {
    double mass[2];       /* sum over bulk nodes of rho per field (RK: per phase) */
    double momentum[3];   /* sum over bulk nodes of rho*u = sum_q f c_q + F/2 */
    double flux_fc[3];    /* sum over bulk nodes of sum_q f c_q (the flux controller's sum) */
    double saturation;    /* RK: mass[0] / (mass[0] + mass[1]); else 0 */
    double max_abs_f;     /* largest |f| over the populations (finite check) */
    int64_t n_bulk;
    int64_t steps_done;
    int32_t nonfinite;    /* 1 if any NaN/Inf population was seen */
} bclbm_stats;

typedef struct {
    double total_ms;        /* CUDA events around the whole block of steps, on the handle's stream */
    double step_kernel_ms;  /* sum over steps of the main step kernel (collide + stream) */
    double density_ms;      /* RK: sum over steps of the density / colour pass (and flux sum) */
    int64_t launches;       /* kernels launched by the call */
    int32_t nsteps;
} bclbm_timing;

typedef struct bclbm_handle bclbm_handle;

int bclbm_create(const bclbm_desc* desc, bclbm_handle** out);
/* Advance nsteps time steps.  The moments of the last step's collision (the
 * values the reference stores in rho/vel during its last node loop) are kept
 * for bclbm_download_macros. */
int bclbm_step(bclbm_handle* h, int nsteps);
/* bclbm_step with CUDA events recorded on the handle's stream around the block
 * and around every launch of the step kernels; synchronises and fills out. */
int bclbm_step_timed(bclbm_handle* h, int nsteps, bclbm_timing* out);
/* Populations after the last step (reference f after swapData + bounce-back),
 * written into the bulk rows of a reference-layout LbField buffer [N*nF*Q];
 * other rows are left untouched. */
int bclbm_download_f(bclbm_handle* h, double* f);
/* rho [N*nF], vel [N*nD], cg [N] (RK only); any may be NULL; bulk rows only. */
int bclbm_download_macros(bclbm_handle* h, double* rho, double* vel, double* cg);
/* The same download in two halves, so the host can write output while the GPU
 * goes on stepping: begin enqueues the copies of the last step's rho / vel / cg
 * into pinned staging on the handle's stream and returns; later bclbm_step calls
 * queue behind the copies; collect waits for the copies only and writes the
 * arrays as bclbm_download_macros does.  One download may be pending at a time. */
int bclbm_macros_begin(bclbm_handle* h);
int bclbm_macros_collect(bclbm_handle* h, double* rho, double* vel, double* cg);
/* FP64 reductions over the current populations (deterministic order). */
int bclbm_reduce(bclbm_handle* h, bclbm_stats* out);
int bclbm_set_force(bclbm_handle* h, const double force[3]);
/* BCLBM_LINKS: the write step's mass flux of the last step, q[phase] = 0.5 * sum of
 * rho u_z over the pressure-boundary nodes (tag bit 16) of fluid phase 1 and 2, in
 * node order (src/std_one_phase/main.cpp:548-562); synchronises */
int bclbm_pressure_flux(bclbm_handle* h, double q[2]);
/* internal node order: out[i] = reference node number of device slot i, [n_bulk] */
int bclbm_node_perm(bclbm_handle* h, int32_t* out);
/* device bytes held by a handle created from desc (admission by HBM footprint) */
int bclbm_footprint(const bclbm_desc* desc, size_t* bytes);
int bclbm_sync(bclbm_handle* h);
/* Frees the handle and its device memory.  The device memory goes back to the
 * library's own stream-ordered pool of the device, which keeps it mapped for the
 * next bclbm_create (no new pages to map); bclbm_trim returns it to the device. */
void bclbm_destroy(bclbm_handle* h);
/* Returns to the devices the memory that destroyed handles left in the library's
 * pools (synchronises each device the library has allocated on; the memory of
 * live handles stays). */
int bclbm_trim(void);
const char* bclbm_error(int status);
const char* bclbm_last_error(const bclbm_handle* h);
/* kernel launches issued by this process since load (for launch accounting) */
int64_t bclbm_launch_count(void);

/* No counterpart in the reference.  The one entry point of this library that
 * allocates nothing.  It is for callers that cannot call cudaMalloc: a host
 * application whose device memory belongs to its own allocator or pool (an
 * allocation behind its back breaks its accounting or its HBM budget), or a
 * latency-critical loop that cannot afford cudaMalloc/cudaFree, which may
 * synchronise the whole device.  Such a caller cannot create a handle, because
 * bclbm_create allocates.
 *
 * It computes the FP64 sums that bclbm_reduce computes - per field
 * sum_q f, sum_q f c_q, and max |f| (+Inf if any value is NaN or Inf) - over a
 * population array the caller holds on the device, in the library's device
 * layout [Q][slot_stride][nfields] (the nfields values of an element side by
 * side; with one field, Q rows of slot_stride values).  precision names the
 * values' format:
 * BCLBM_F64 = plain FP64 values of f (the device format of handles created
 * with BCLBM_FLAG_EXACT or BCLBM_FLAG_FP64_FMA; a default BCLBM_F64 handle keeps
 * int64 fixed point on the device, which this entry point does not read); the
 * shifted formats as described at BCLBM_F32..BCLBM_BF16, with rho_ref and
 * store_scale as given to bclbm_create, 0 meaning the default (F16: 4096).
 * d_out: caller-allocated device buffer of 6 doubles,
 *   [mass0, mass1, flux_x, flux_y, flux_z, max|f|].
 * stream: a cudaStream_t, or NULL for the default stream; the call is
 * asynchronous on that stream.
 *
 * The only scratch (per-block partial sums) is a fixed device array inside
 * the library, 1.5 MiB, held by every GPU that loads the library until the
 * process exits.  n_slots above BCLBM_STATIC_MAX_SLOTS is rejected with
 * BCLBM_ERR_INVALID and a message on stderr.  All calls share that array:
 * calls whose kernels overlap on the GPU race and give wrong sums, so order
 * them on one stream.  The first call in a CUDA context (normally the device's
 * primary context) looks up the array's device address with that context
 * current and keeps it for that context; make that first call before any
 * stream capture.  After cudaDeviceReset the next call runs in a new context
 * and looks the address up again.  An error already pending on the calling
 * thread is returned (BCLBM_ERR_CUDA) without launching and is not cleared. */
#define BCLBM_STATIC_MAX_SLOTS 8388608
int bclbm_moments_static(int32_t lattice_q, int32_t precision, int32_t nfields, int32_t n_slots,
                         int32_t slot_stride, const void* d_pops, double rho_ref, double store_scale,
                         double* d_out, void* stream);

/* ---------------------------------------------------------------------------
 * Lattice builder: a voxel mask to the arrays bclbm_desc takes.  The
 * reference builds them in Python (PythonScripts/vtklb.py writes a .vtklb
 * file, src/lbsolver/LBgrid.h and LBnodes.h read it); this restates the
 * single-rank numbering of vtklb.py:6-45, 84-114, 182-218 and
 * Nodes::setupNodeType (LBnodes.h:141-209) on the host cores.
 * mask: [shape[0]*...*shape[nd-1]] in C order (x slowest), 1 fluid, 0 solid.
 * periodic: bit d set for a periodic axis d (x = 1, y = 2, z = 4).
 * The result holds neigh [N*Q], types [N] and pos [N*nD] (-1 for node 0) with
 * N = 1 + n_fluid + n_solid; the bulk list is nodes 1..n_fluid.
 * ------------------------------------------------------------------------- */
typedef struct bclbm_lattice bclbm_lattice;

int bclbm_lattice_build(int32_t lattice_q, int32_t nd, const int32_t* shape, const int8_t* mask,
                        uint32_t periodic, bclbm_lattice** out);
int bclbm_lattice_info(const bclbm_lattice* lat, int64_t* n_nodes, int64_t* n_fluid, int64_t* n_solid);
/* copies the arrays out (any pointer may be NULL) */
int bclbm_lattice_export(const bclbm_lattice* lat, int32_t* neigh, int16_t* types, int32_t* pos);
void bclbm_lattice_free(bclbm_lattice* lat);
/* The same object from a .vtklb file as PythonScripts/vtklb.py writes it and
 * LBvtk/Grid/Nodes read it (src/lbsolver/LBvtk.h:221-662, LBgrid.h:127-148,
 * LBnodes.h:112-209): one rank (no PROCESSOR blocks), text (an ASCII or BINARY
 * header, both read as text as LBvtk does), 64-bit offsets (no 2 GiB limit).  Node types follow Nodes::setupNodeType from the nodetype
 * attribute; the bulk list is the nodes of type 2 and 3. */
int bclbm_lattice_read_vtklb(const char* path, int32_t lattice_q, bclbm_lattice** out);
/* a SCALARS attribute of the file by name, [N] doubles (0 at the ghost node) */
int bclbm_lattice_attribute(const bclbm_lattice* lat, const char* name, double* out);

/* ---------------------------------------------------------------------------
 * Multi-instance batch (continuous batching of many solves on one GPU).  No
 * counterpart in the reference, whose executables run one geometry per
 * process; it serves many independent geometries, each one the reference's
 * std_case time loop (src/std_case/main.cpp:110-145) over its own lattice.
 *
 * A batch holds up to max_instances single-phase instances of one lattice,
 * collision and precision (BGK or TRT; F64 fixed-point or FMA, or a shifted
 * storage format; BCLBM_FLAG_EXACT is BCLBM_ERR_UNSUPPORTED).  Each instance is
 * built from an ordinary bclbm_desc, as bclbm_create builds a handle.  All
 * instances advance together: one persistent kernel per step walks the
 * concatenated list of every instance's 256-node blocks, and a block of
 * steps_per_graph steps is captured once as a CUDA graph and replayed (0: no
 * graph).  Instances are admitted and retired between steps without
 * re-capturing.  Each instance's populations, moments and sums are
 * bit-identical to a handle created from the same descriptor and stepped the
 * same number of times, whatever else is in the batch.
 * ------------------------------------------------------------------------- */
typedef struct bclbm_batch bclbm_batch;

int bclbm_batch_create(int32_t lattice_q, int32_t collision, int32_t precision, uint32_t flags,
                       int32_t max_instances, size_t hbm_budget, int32_t steps_per_graph, bclbm_batch** out);
/* Admission by HBM footprint: BCLBM_ERR_BUDGET (nothing allocated) if the
 * instance's bclbm_footprint would take the batch above hbm_budget or no slot
 * is free.  *id receives the instance id (its slot).  Admission takes the
 * instance's first time step (the one that reads the initial populations), so
 * its steps_done is 1 on return. */
int bclbm_batch_admit(bclbm_batch* b, const bclbm_desc* desc, int32_t* id);
/* bclbm_batch_admit taking first_steps >= 1 steps with the single-instance
 * kernel before the instance joins (steps_done = first_steps on return); used
 * to keep the parity of a solve's step count when it moves between batches. */
int bclbm_batch_admit_steps(bclbm_batch* b, const bclbm_desc* desc, int32_t first_steps, int32_t* id);
/* Admission of a handle the caller created (bclbm_create + bclbm_step, e.g. on
 * another host thread while the batch runs): on BCLBM_OK the batch owns h and
 * destroys it at retirement; on any error h stays the caller's.  h must match
 * the batch's lattice, collision and precision and have taken >= 1 step. */
int bclbm_batch_attach(bclbm_batch* b, bclbm_handle* h, int32_t* id);
/* Frees the instance and its HBM; its id may be reused by a later admission. */
int bclbm_batch_retire(bclbm_batch* b, int32_t id);
/* Advances every admitted instance by nsteps steps (asynchronous). */
int bclbm_batch_step(bclbm_batch* b, int32_t nsteps);
/* bclbm_reduce's sums for n instances (synchronises); steps_done is per instance. */
int bclbm_batch_stats(bclbm_batch* b, int32_t n, const int32_t* ids, bclbm_stats* out);
/* bclbm_download_f of one instance (synchronises). */
int bclbm_batch_download_f(bclbm_batch* b, int32_t id, double* f);
/* device bytes held by the admitted instances, their number, steps taken by the batch */
int bclbm_batch_info(bclbm_batch* b, size_t* used_bytes, int32_t* n_active, int64_t* steps);
int bclbm_batch_sync(bclbm_batch* b);
const char* bclbm_batch_last_error(const bclbm_batch* b);
void bclbm_batch_destroy(bclbm_batch* b);

/* ---------------------------------------------------------------------------
 * VTU output of the reference's write step: Output<LT, T, FMT>
 * (src/io/Output.h:26-177) over VTK::Output (src/io/VTK.h:1421-1550).  The
 * files are byte-identical to the reference's for the same positions,
 * variables and write sequence (only the PVTU "Created" time differs):
 * <dir>/<name>_<n:7>.pvtu and <dir>/vtu/<rank:4>_<name>_<n:7>.vtu, one voxel
 * (pixel in 2-D) per cell.  Where the appended data would pass 2^31 bytes
 * (the reference's int offsets overflow there) the VTU is written with
 * header_type="UInt64".
 *
 * create: the cells are the written nodes; pos [n_cells*nd] their positions
 *   (Grid::pos(nodes), LBgrid.h:114); nodes [n_cells] their node numbers (for
 *   bclbm_output_add_field), or NULL for arrays only (the
 *   Output(pos, dir, rank, nproc, ...) form).  value_type: the on-disk type T;
 *   format: BCLBM_VTU_BINARY (the reference's default), BCLBM_VTU_ASCII, or
 *   BCLBM_VTU_BINARY64 (64-bit counts and offsets whatever the size).
 *   Creates <dir> and <dir>/vtu as the reference does (mkdir of each, 0700).
 *   nproc > 1 is BCLBM_ERR_UNSUPPORTED (the PVTU pieces of several ranks share
 *   one file through MPI-IO).
 * add_file: Output::add_file (Output.h:63).
 * add_field: Output::add_variables for one ScalarField (dim 1) or VectorField
 *   (dim nD) of n_fields fields in the reference layout (LBfield.h:69, 219):
 *   field_no -1 adds one variable per field (Output.h:80-88); field_no >= 0
 *   adds that field alone (add_variable_with_names, Output.h:111-126).  As in
 *   the reference, the name gets the field number appended (name<i>) whenever
 *   n_fields > 1.
 * add_array: Output::add_variables for a plain vector of `length` values of
 *   data_type (contiguous; components per cell = length / n_cells).
 * The data pointers are kept and read at each write (the reference keeps
 * references to its fields).
 * write: Output::write(time) (Output.h:58).  write_async: reads the values
 *   now, writes the files on a background thread and returns; the next call on
 *   the object, or bclbm_output_wait, waits for it and returns its status.
 * ------------------------------------------------------------------------- */
#define BCLBM_VTU_FLOAT64 0
#define BCLBM_VTU_FLOAT32 1
#define BCLBM_VTU_INT32 2
#define BCLBM_VTU_BINARY 0   /* appended raw, 32-bit counts (64-bit past 2^31 bytes) */
#define BCLBM_VTU_ASCII 1
#define BCLBM_VTU_BINARY64 2 /* appended raw with header_type="UInt64" at any size */
typedef struct bclbm_output bclbm_output;

int bclbm_output_create(int32_t nd, int64_t n_cells, const int32_t* pos, const int32_t* nodes, const char* dir,
                        int32_t rank, int32_t nproc, int32_t value_type, int32_t format, bclbm_output** out);
int bclbm_output_add_file(bclbm_output* o, const char* name);
int bclbm_output_add_field(bclbm_output* o, const char* name, const double* data, int32_t n_fields, int32_t dim,
                           int32_t field_no);
int bclbm_output_add_array(bclbm_output* o, const char* name, const void* data, int32_t data_type, int64_t length);
int bclbm_output_write(bclbm_output* o, double time);
int bclbm_output_write_async(bclbm_output* o, double time);
int bclbm_output_wait(bclbm_output* o);
int bclbm_output_info(const bclbm_output* o, int64_t* n_points, int64_t* n_cells, int32_t* n_files);
const char* bclbm_output_last_error(const bclbm_output* o);
void bclbm_output_destroy(bclbm_output* o);

#ifdef __cplusplus
}
#endif
#endif
