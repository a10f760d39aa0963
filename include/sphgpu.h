/*
 * sphgpu.h -- C ABI of the GB300 (sm_103a) neighbour search and pair loop
 * that replaces SmoothedParticles.jl's cell-list / pair-loop layer.
 *
 * One handle = one ParticleSystem on one GPU.  Particle state lives in device
 * memory as struct-of-arrays between calls; the handle owns one CUDA stream
 * and every call is ordered on it.  Host arrays passed in or out are always in
 * the reference's particle order (the index of a particle in sys.particles);
 * inside the device the particles are kept sorted by cell.
 *
 * Every function returns an int status: SPH_OK (0) or a negative SPH_ERR_*.
 * sph_last_error() gives a message for the last failure on a handle.  A handle
 * must not be used from two threads at once; separate handles are independent.
 * Operators are the built-in ones (SPH_OP_*): arbitrary Julia closures have no
 * device counterpart and there is no CPU fallback.
 *
 * Reference paths below are relative to the SmoothedParticles.jl project.
 */
#ifndef SPHGPU_H
#define SPHGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPHGPU_ABI_VERSION 2

/* ---- status codes */
#define SPH_OK 0
#define SPH_ERR_ARG -1         /* invalid argument (null pointer, bad op, size)    */
#define SPH_ERR_CUDA -2        /* a CUDA runtime call failed                       */
#define SPH_ERR_STATE -3       /* call out of order (e.g. pair pass on stale cells) */
#define SPH_ERR_NOMEM -4       /* device allocation failed                         */
#define SPH_ERR_DEVICE -5      /* a kernel reported an error (bounds, overflow)    */
#define SPH_ERR_UNSUPPORTED -6 /* operator / mode combination not provided         */
#define SPH_ERR_TIMEOUT -7     /* a bounded device wait gave up                    */
#define SPH_ERR_BUDGET -8      /* request does not fit the memory budget          */

/* ---- particle types (the `type` field of the reference's examples) */
#define SPH_FLUID 0
#define SPH_WALL 1

/* ---- precision of the pair passes */
#define SPH_PREC_FP64 0  /* FP64 throughout; bit-exact with the CPU restatement */
#define SPH_PREC_MIXED 1 /* FP32 pair arithmetic on cell-relative positions,
                            FP64 positions, integration and accumulators      */

/* ---- built-in binary (pair) operators: apply!(sys, op!; self) */
#define SPH_OP_DENSITY 1       /* rho_p     += m W(r_pq); fluid p, every q         */
#define SPH_OP_DENSITY_REF 2   /* rho_ref_p += m W(r_pq); fluid p, every q         */
#define SPH_OP_FORCE 3         /* fluid p: a_p += pressure (+ Monaghan viscosity
                                  between fluid particles); xsph_p += sum over
                                  fluid q of wx (v_q - v_p), wx = m W / rho_bar,
                                  formed (FP64) as sum wx v_q - v_p sum wx */
#define SPH_OP_WALL_PRESSURE 4 /* wall p: P_p = (sum P_q W + sum rho_q (g.x_pq) W)
                                  / sum W over fluid q (Adami et al. 2012)       */
/* ---- built-in unary operators: apply!(sys, op!) */
#define SPH_OP_RESET_RHO 10
#define SPH_OP_RESET_RHO_REF 11
#define SPH_OP_RESET_A 12     /* a = 0 and xsph = 0                            */
#define SPH_OP_EOS 13         /* the system's EOS (sph_params.eos), fluid p:
                                 Tait P = B((rho/rho_ref)^7 - 1), P/rho^2; or
                                 linear P = c0^2 (rho - rho_ref), P/rho0^2     */
#define SPH_OP_KICK 14        /* v += dt/2 (a + g)  (fluid)                    */
#define SPH_OP_DRIFT 15       /* x += dt (v + eps xsph)  (fluid)               */
#define SPH_OP_HYDROSTATIC 16 /* rho_ref /= (1 + rho0 g (H_col - y) / B)^(1/7) */

/* ---- functions for sum(sys, func, x) / sum(sys, func, p) */
#define SPH_SUM_DENSITY 1  /* m W(r) over all q                      */
#define SPH_SUM_KERNEL 2   /* W(r) over all q                        */
#define SPH_SUM_PRESSURE 3 /* (m / rho_q) P_q W(r) over fluid q      */
#define SPH_SUM_SHEPARD 4  /* (m / rho_q) W(r) over fluid q          */

/* ---- fields for sph_get_field / sph_set_field */
#define SPH_FIELD_X 1       /* double[n][3]                                   */
#define SPH_FIELD_V 2       /* double[n][3]                                   */
#define SPH_FIELD_A 3       /* double[n][3]                                   */
#define SPH_FIELD_XSPH 4    /* double[n][3]                                   */
#define SPH_FIELD_RHO 5     /* double[n]                                      */
#define SPH_FIELD_RHO_REF 6 /* double[n]                                      */
#define SPH_FIELD_P 7       /* double[n]; setting P also sets P/rho^2 (set RHO first) */
#define SPH_FIELD_TYPE 8    /* int32[n]                                       */
#define SPH_FIELD_OID 9     /* int64[n] index at upload time (read only)      */
#define SPH_FIELD_KEY 10    /* int64[n] cell key of the last binning (read only) */

/* Physical and geometric parameters of one system. */
typedef struct sph_params {
  int32_t dim;           /* 2 or 3: kernel normalisation and stored components */
  int32_t precision;     /* SPH_PREC_FP64 or SPH_PREC_MIXED                    */
  double h;              /* neighbour radius = kernel support (the reference's h) */
  double domain_min[3];  /* bounding box of the domain (structs.jl:63)          */
  double domain_max[3];
  double mass;           /* particle mass m                                     */
  double rho0;           /* reference density                                   */
  double c0;             /* numerical speed of sound; Tait B = c0^2 rho0 / 7     */
  double h_smooth;       /* smoothing length in the viscosity regulariser        */
  double alpha;          /* artificial viscosity coefficient                     */
  double eps_xsph;       /* XSPH coefficient                                     */
  double gravity[3];
  double dt;
  double col_height;     /* free-surface height for SPH_OP_HYDROSTATIC           */
  int32_t vertical_axis; /* 0-based axis along gravity                           */
  int32_t eos;           /* SPH_EOS_TAIT (0) or SPH_EOS_LINEAR (1), below         */
  double cell_factor;    /* cell size / h: 0 or 1 = the reference's cells of size h
                            (structs.jl:66-68); SPH_PREC_MIXED systems accept
                            1..2 (the pair set does not depend on it; the
                            neighbour order and the FP32 sums do).  A mixed
                            system's grid is also offset by 5/16 of a cell
                            along each of its axes (sph_geometry reports its
                            keys).  No reference counterpart; ABI version 2. */
} sph_params;

/* Equation of state of SPH_OP_EOS and of the step's fused EOS, and the
 * pressure term P/rho^2 the force pass uses:
 *   SPH_EOS_TAIT    P = B((rho/rho_ref)^7 - 1), B = c0^2 rho0 / 7; P/rho^2
 *                   (the weakly compressible dam-break scheme)
 *   SPH_EOS_LINEAR  P = c0^2 (rho - rho_ref); P/rho0^2 -- find_pressure! and
 *                   internal_force! of tests/test_collision_2d.jl:71-78 */
#define SPH_EOS_TAIT 0
#define SPH_EOS_LINEAR 1

typedef struct sph_system sph_system;

/* ParticleSystem(T, domain, h) -- structs.jl:57-92.  Computes key_phase,
 * key_lim, key_max, key_diff from the domain's bounding box and allocates the
 * dense cell table on device `device`. */
int sph_create(const sph_params* params, int device, sph_system** out);
int sph_destroy(sph_system* sys);
const char* sph_last_error(const sph_system* sys);
int sph_abi_version(void);

/* Geometry of the cell table (structs.jl:66-82): key_phase[3], key_lim[3],
 * key_max, key_diff[27] (first n_diff used, in the reference's order). */
int sph_geometry(const sph_system* sys, int64_t key_phase[3], int64_t key_lim[3],
                 int64_t* key_max, int64_t key_diff[27], int32_t* n_diff);

/* generate_particles! (grids.jl:253-258): replaces the particle set with n
 * particles given in the reference's order.  x, v: n x 3 doubles (v may be
 * NULL = 0); rho, rho_ref may be NULL (= 0); type may be NULL (= fluid).
 * In 2D every z must be 0 (the reference's Rectangle has x3 in [0, 0]). */
int sph_upload(sph_system* sys, int64_t n, const double* x, const double* v,
               const double* rho, const double* rho_ref, const int32_t* type);
int sph_num_particles(sph_system* sys, int64_t* n);
/* ParticleField (structs.jl:118-125) as whole-array copies in reference order. */
int sph_get_field(sph_system* sys, int field, void* host_out);
int sph_set_field(sph_system* sys, int field, const void* host_in);

/* create_cell_list! -- core.jl:51-90.  Removes particles outside the domain's
 * bounding box (NaN included) with the reference's tail-fill compaction, bins
 * the rest by cell key (counting sort + per-cell descending-index order) and
 * reorders the device arrays by cell. */
int sph_create_cell_list(sph_system* sys);

/* apply!(sys, op!; self) -- core.jl:151-161 with a built-in operator; a pair
 * operator runs _apply_binary! (core.jl:94-112) for every particle and, if
 * self != 0, the self term op!(p, p, 0.0) after the neighbours. */
int sph_apply(sph_system* sys, int op, int self);
/* apply_unary! -- core.jl:138-142 with a built-in unary operator. */
int sph_apply_unary(sph_system* sys, int op);

/* sum(sys, func, x) -- core.jl:240-260, at nq points (x: nq x 3 doubles). */
int sph_sum_point(sph_system* sys, int func, int64_t nq, const double* x, double* out);
/* sum(sys, func, p) -- core.jl:271-291, for particles by reference index. */
int sph_sum_particle(sph_system* sys, int func, int64_t nq, const int64_t* index,
                     double* out);

/* One verlet_step! (examples/collapse_symplectic.jl:170-180) per step: kick,
 * drift, create_cell_list!, density sum with self term, Tait EOS, wall
 * pressure, force, kick; the kick + drift run inside the binning's key kernel
 * and the EOS inside the density pass.  From four steps per call (and with
 * per-kernel timing off) the steps replay a CUDA graph of two steps captured
 * on first use and kept until the system's buffers, particle count or tuning
 * change; the results are those of single steps. */
int sph_step(sph_system* sys, int nsteps);

/* One step with its host input and output, for a caller that keeps the
 * particle state on the host between steps (no reference counterpart: the
 * field reads and writes around a verlet_step! of a Julia time loop, in one
 * call).  Sets the nin fields in_fields[i] from in[i] (as sph_set_field),
 * takes one step (as sph_step(sys, 1)) and reads the nout fields
 * out_fields[i] into out[i] (as sph_get_field, the count after the step's
 * removals).  Each read starts on a second stream as soon as its field is
 * final within the step -- positions, reference density, type, indices and
 * keys after the binning, density and pressure after the wall pressure, the
 * rest at the end -- so that its gather and copy overlap the step's
 * remaining passes; reads into pageable memory all wait for the end. */
int sph_step_io(sph_system* sys, int nin, const int32_t* in_fields, const void* const* in,
                int nout, const int32_t* out_fields, void* const* out);
/* Initial state of the dam break (collapse_symplectic.jl:186-191 plus the
 * hydrostatic reference density): bin, rho_ref sum, hydrostatic scaling,
 * density sum, EOS, wall pressure, force. */
int sph_init_state(sph_system* sys);

/* Pair interactions evaluated since the last reset: ordered pairs (p, q),
 * p != q, r_pq <= h, counted per pair pass over the targets the pass's
 * operator acts on (fluid targets; wall targets for the wall pressure).  This
 * is the reference's action! call count (core.jl:105-108) without the calls
 * on targets the operator ignores. */
int sph_pair_count(sph_system* sys, uint64_t* pairs, int reset);
/* Hits evaluated per category since the last reset (no reference counterpart;
 * used to count algorithmic flops): [0] density sums, [1] wall pressure (fluid
 * neighbours), [2] force fluid-fluid, [3] force fluid-wall, [4] force pairs
 * with the viscosity term active; [5..7] unused. */
int sph_pair_stats(sph_system* sys, uint64_t counts[8], int reset);
/* Blocks until all work queued on the handle's stream is done and reports any
 * device-side error flag. */
int sph_synchronize(sph_system* sys);
/* The handle's CUDA stream (a cudaStream_t), for callers that time or order
 * their own work against it. */
int sph_stream(sph_system* sys, void** stream);

/* ---- diagnostics (no reference counterpart) */
/* Cell key per particle (reference order) and every ordered neighbour pair in
 * the reference's traversal order (target ascending; key_diff order;
 * descending neighbour index), as (p, q) reference indices.  Writes up to cap
 * pairs and the total count to *count. */
int sph_debug_pairs(sph_system* sys, int64_t* pairs, int64_t cap, int64_t* count);
/* The ordered pairs (p, q) the last density pass (SPH_OP_DENSITY or
 * SPH_OP_DENSITY_REF) acted on, read back from what that pass stored for the
 * force pass of the same cells -- the FP64 path's rows or the mixed path's
 * hit masks -- as reference indices, fluid targets only, each target's
 * neighbours in the reference's traversal order (targets ascending).  The
 * mixed path's pair set is checked through this against the oracle.
 * SPH_ERR_STATE when no density pass ran since the last binning or a
 * target's hits were not stored (an overflow sent it to the traversal). */
int sph_debug_hits(sph_system* sys, int64_t* pairs, int64_t cap, int64_t* count);
/* Per-kernel timing with CUDA events on the handle's stream, enabled by
 * sph_set_profiling(sys, 1).  kernel ids are SPH_KERNEL_*. */
#define SPH_KERNEL_BIN_KEYS 0
#define SPH_KERNEL_BIN_REMOVE 1
#define SPH_KERNEL_BIN_SCAN 2
#define SPH_KERNEL_BIN_SCATTER 3
#define SPH_KERNEL_BIN_RANK 4
#define SPH_KERNEL_BIN_GATHER 5
#define SPH_KERNEL_DENSITY 6
#define SPH_KERNEL_FORCE 7
#define SPH_KERNEL_UNARY 8
#define SPH_KERNEL_SUM 9
#define SPH_KERNEL_IO 10
#define SPH_KERNEL_WALL 11
#define SPH_KERNEL_COUNT 12
int sph_set_profiling(sph_system* sys, int on);
int sph_kernel_stats(sph_system* sys, int kernel, double* total_ms, int64_t* launches);
int sph_reset_kernel_stats(sph_system* sys);
/* Kernels launched by this handle since creation. */
int sph_launch_count(sph_system* sys, int64_t* launches);
/* ---- tuning (no reference counterpart): warps per block of the pair passes
 * (2, 4 or 8, i.e. 64/128/256 threads; default 4).  Results do not depend on
 * it; the batched ensemble's autotuner picks it per size class. */
int sph_set_tuning(sph_system* sys, int warps_per_block);
int sph_get_tuning(const sph_system* sys, int* warps_per_block);
/* Threads per cell chunk of the mixed-precision pair passes (no reference
 * counterpart): 32, 64 or 128 threads share one work item (<= 32 targets of
 * one cell), each warp taking every 1st, 2nd or 4th 32-candidate chunk of the
 * neighbour sequence, their FP64 sums added in warp order (default 32).  The
 * mixed results depend on it at the FP32 level (the batches of each lane's
 * FP32 sums change), bit-exactly reproducibly for a given setting; the FP64
 * path ignores it.  The batched ensemble's autotuner picks it per size class. */
int sph_set_chunk_threads(sph_system* sys, int threads);
int sph_get_chunk_threads(const sph_system* sys, int* threads);

/* ---- assemble_matrix / assemble_vector (src/core.jl:164-225) on the device
 * and the conjugate-gradient solve of the implicit example
 * (examples/collapse_dry_implicit.jl:218-233).  The matrix has one entry per
 * pair within the support, the diagonal (q = p, r = 0) included, rows and
 * columns in reference particle order, as CSR with each row's columns
 * ascending.  Built-in functions:
 *   SPH_MAT_KERNEL      A_pq = W(r_pq)
 *   SPH_MAT_PROJECTION  the ISPH projection matrix of
 *                       collapse_dry_implicit.jl:151-160 with this library's
 *                       kernel: A_pq = 2 h^2 (m / rho0) rDW(r_pq) for q != p,
 *                       A_pp = h^2 L_p (+ param * max(lambda_p, 0) for fluid p,
 *                       param = C_free), L_p and lambda_p the div_L_lambda!
 *                       sums (collapse_dry_implicit.jl:140-145); h = support
 *   SPH_VEC_PROJECTION  b_p = -h^2 div_p / dt (collapse_dry_implicit.jl:162-164)
 * sph_cg: unpreconditioned CG from x = 0 until ||r|| <= reltol ||b|| or
 * maxiter iterations (maxiter < 0: n), host arrays in reference order. */
#define SPH_MAT_KERNEL 1
#define SPH_MAT_PROJECTION 2
#define SPH_VEC_PROJECTION 1
typedef struct sph_csr sph_csr;
int sph_assemble_matrix(sph_system* sys, int func, double param, sph_csr** out);
int sph_assemble_vector(sph_system* sys, int func, double* out);
int sph_csr_info(const sph_csr* a, int64_t* n, int64_t* nnz);
int sph_csr_download(sph_csr* a, int64_t* row_ptr, int32_t* col, double* val);
int sph_csr_destroy(sph_csr* a);
int sph_cg(sph_csr* a, const double* b, double* x, double reltol, int32_t maxiter,
           int32_t* iters, double* resid);

/* ---- ParaView export: new_pvd_file / save_frame! / save_pvd_file
 * (src/IO.jl:15-75).  sph_vtk_open creates `dir` (mkpath) and a frame series;
 * sph_vtk_save_frame gathers the positions plus the fields in `fields` (bit
 * 1 << SPH_FIELD_*) on the system's stream, in reference particle order, and
 * returns: the copy to pinned host memory runs on a separate stream and a host
 * thread writes <dir>/frame<k>.vtp (VTK XML PolyData, raw appended binary,
 * one vertex cell per particle); at most two frames are in flight (a third
 * call waits for a slot).  *frame (optional) = k.  sph_vtk_close waits for
 * every frame and writes <dir>/result.pvd with the frames' `time` values.
 * No reference counterpart for sph_vtk_frames (frames on disk so far). */
typedef struct sph_vtk sph_vtk;
int sph_vtk_open(sph_system* sys, const char* dir, sph_vtk** out);
int sph_vtk_save_frame(sph_vtk* vtk, unsigned fields, double time, int32_t* frame);
int sph_vtk_frames(sph_vtk* vtk, int32_t* written);
int sph_vtk_close(sph_vtk* vtk);

/* ---- device-side particle generation: covering(grid, shape) of
 * src/grids.jl:52-66 / :128-144 (square / cubic grid, points i*dr in the
 * reference's loop order, i outer) for a Box / Rectangle (src/geometry.jl:15-43)
 * or a BoundaryLayer (src/geometry.jl:198-234) with an optional Specification
 * x[keep_axis] < keep_max (src/geometry.jl:179-196).  2D shapes have
 * lo[2] = hi[2] = 0. */
#define SPH_SHAPE_BOX 1
#define SPH_SHAPE_LAYER 2
typedef struct sph_shape {
  int32_t kind;        /* SPH_SHAPE_BOX or SPH_SHAPE_LAYER                      */
  int32_t type;        /* SPH_FLUID / SPH_WALL of the generated particles       */
  double dr;           /* grid spacing                                           */
  double lo[3], hi[3]; /* the box (BOX: the filled shape; LAYER: the enclosed box) */
  double width;        /* LAYER: width of the layer                              */
  int32_t keep_axis;   /* LAYER: keep points with x[keep_axis] < keep_max; -1: all */
  int32_t reserved;
  double keep_max;
} sph_shape;
/* Replaces the particle set by the particles of shapes[0..count) in order (as
 * generate_particles! once per shape, src/grids.jl:253-258), generated on the
 * device: v = 0, rho = rho_ref = 0.  Same result as sph_upload of the same
 * points; *n_out = the particle count. */
int sph_generate(sph_system* sys, const sph_shape* shapes, int count, int64_t* n_out);
/* The particle count sph_generate would produce for a system of dimension dim,
 * computed on `device` without a system (for admission before allocation). */
int sph_shape_count(int device, int dim, const sph_shape* shapes, int count, int64_t* n_out);

/* ---- device memory accounting for admission by an HBM budget (no
 * reference counterpart).  sph_memory_estimate: the device bytes a system
 * with these parameters holds once it stores n particles (cell tables plus the
 * particle arena; sum() query buffers excluded), computed on the host without
 * any CUDA call.  sph_memory_usage: the bytes the system holds now.
 * sph_query: *idle = 1 when all work queued on the system's stream has
 * finished, 0 otherwise (never waits). */
int sph_memory_estimate(const sph_params* params, int64_t n, uint64_t* bytes);
int sph_memory_usage(const sph_system* sys, uint64_t* bytes);
int sph_query(sph_system* sys, int* idle);
/* The temporary device bytes sph_generate / sph_shape_count allocate (and
 * free before returning) for these shapes: one word per point of the largest
 * shape's bounding lattice plus scan scratch; host arithmetic only. */
int sph_generate_scratch(int dim, const sph_shape* shapes, int count, uint64_t* bytes);
/* cudaMemGetInfo of `device`: the bytes free and in total (what a server
 * compares its admitted budget with). */
int sph_device_memory(int device, uint64_t* free_bytes, uint64_t* total_bytes);

/* ---- batched ensembles (no reference counterpart)
 *
 * A batch steps many independent systems (same device) together.  The first
 * sph_batch_step of two or more steps captures every member's fused step
 * (the sph_step sequence) into one CUDA graph, two steps per graph, each
 * member an independent branch; every further pair of steps is one graph
 * launch, and the branches overlap on the device.  An odd last step runs on
 * the members' own streams.  Each member's results are bit-identical to
 * stepping it alone.  The graph is captured again when a member's buffers,
 * particle set (sph_upload, sph_generate) or tuning changed, or when an odd
 * number of steps taken outside the graph left a member on the other half of
 * its ping-pong buffers; members must outlive the batch and must not be
 * stepped by other calls while a batch step is in flight. */
typedef struct sph_batch sph_batch;
int sph_batch_create(sph_system* const* members, int count, sph_batch** out);
int sph_batch_destroy(sph_batch* batch);
const char* sph_batch_last_error(const sph_batch* batch);
int sph_batch_step(sph_batch* batch, int nsteps);
int sph_batch_synchronize(sph_batch* batch);
/* Fused steps (default when every member is mixed precision and of one
 * dimension): each kernel of the step is one launch over all members, so a
 * graph holds ~44 kernels for two steps whatever the member count; off: one
 * graph branch per member.  Results are the same either way. */
int sph_batch_set_fused(sph_batch* batch, int on);
/* Warps per block (2, 4 or 8) of the fused pair passes; without fused steps
 * each member's own sph_set_tuning applies.  Results do not depend on it. */
int sph_batch_set_tuning(sph_batch* batch, int warps_per_block);
/* kernels in one captured graph, graph launches so far, kernels executed */
int sph_batch_stats(sph_batch* batch, int64_t* kernels_per_graph, int64_t* graph_launches,
                    int64_t* kernels);
/* the stream the graph is launched on (a cudaStream_t) */
int sph_batch_stream(sph_batch* batch, void** stream);
/* *idle = 1 when everything queued by the batch and by its members has
 * finished, 0 otherwise (never waits). */
int sph_batch_query(sph_batch* batch, int* idle);

/* ---- allocation-free cell-list build (no counterpart in the reference)
 *
 * For callers that must not have the library allocate device memory: a host
 * whose GPU memory is owned by its own pool or budget (CUDA.jl's allocator, a
 * serving process that admits work against a fixed HBM budget) cannot let a
 * library cudaMalloc behind its back -- the allocation escapes the pool's
 * accounting, may fail mid-run, and cudaMalloc/cudaFree synchronise the
 * device.  sph_cell_list_noalloc allocates nothing.  Its scratch is one
 * static device array of about 21 MB that every GPU which loads the library
 * holds until the process exits; every call shares it, so calls that overlap
 * on the GPU (different streams, or concurrent host threads) race.  The first
 * call in a CUDA context looks up the array's device address
 * (cudaGetSymbolAddress) with that context current and caches it under the
 * context's id; make that first call before any stream capture.  A context
 * destroyed and created again (cudaDeviceReset) is a new context: its first
 * call looks the address up again, so it too must come before any capture.
 *
 * Inputs: params (dim, h and domain_min/max are used; the same checks as
 * sph_create), n particles, d_x = device
 * array of n x 3 doubles.  Outputs (device memory owned by the caller):
 * d_cell_start[key_max + 2] and d_order[n].  Cell k (1-based key as in
 * find_key) holds d_order[d_cell_start[k] .. d_cell_start[k+1]), particle
 * indices in descending order, as create_cell_list! builds its cells when no
 * particle is removed.  Particles outside the domain's bounding box (NaN
 * included) are not binned; they follow in d_order[d_cell_start[key_max+1]
 * .. n), in descending index order.  Work is queued on `stream` (a
 * cudaStream_t; NULL = default stream) and the call returns without waiting.
 * Returns SPH_ERR_BUDGET if n > SPH_NOALLOC_MAX_PARTICLES or key_max >
 * SPH_NOALLOC_MAX_CELLS. */
#define SPH_NOALLOC_MAX_PARTICLES (1 << 20)
#define SPH_NOALLOC_MAX_CELLS (1 << 20)
int sph_cell_list_noalloc(const sph_params* params, int64_t n, const double* d_x,
                          int32_t* d_cell_start, int32_t* d_order, void* stream);

/* Issue-rate microbenchmark of one arithmetic pipe on `device` (no reference
 * counterpart; the roofline denominators of the pair passes):
 * which = 0 FP64 FMA, 1 FP32 FMA, 2 FP64 add, 3 int64 -> FP64 conversion,
 * 4 FP64 FMA with a conversion beside each (FMA rate).  Returns
 * thread-instructions/s. */
int sph_pipe_peak(int device, int which, double* instr_per_s);

/* Diagnostics (no reference counterpart): the FP64 arithmetic the pair passes
 * form on the integer pipes, applied on `device` to n host values, for tests
 * against the IEEE operations.  op 0: a[i] - b[i] through fixed-point copies
 * at scale 2^k (the FP64 subtraction when a value has no exact copy);
 * 1: sqrt(a[i]); 2: 1 / a[i]; 3: 2 / a[i].  out[i] receives the result. */
int sph_arith_check(int device, int op, int k, int n, const double* a, const double* b,
                    double* out);

#ifdef __cplusplus
}
#endif
#endif
