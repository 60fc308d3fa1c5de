/*
 * lbgb -- C ABI of the GB300 D2Q9 lattice-Boltzmann library (liblbgb.so).
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (cudaStream_t passed as void*; NULL = legacy default stream), launches
 * asynchronously on that stream and returns 0 on success or a negative
 * LBGB_E* code.  Nothing here allocates device memory: the caller owns every
 * buffer (arrays, workspaces).  A message for the last failure on the calling
 * host thread is available from lbgb_last_error().
 *
 * Population layout: channel-major structure of arrays, f[i * chan_stride + c]
 * with cell c = k * ny + l (k = x index, l = y index, l fastest), i.e. a
 * C-contiguous (9, nx, ny) array -- the layout of the reference's f_ikl
 * (simulators/parallel_lid_drive_cavity/cavity_opt1.py:74-82) and of the
 * (9, N) view its native kernels take (c/d2q9.h:38-39).
 * Channel order: 0, E(1,0), N(0,1), W(-1,0), S(0,-1), NE(1,1), NW(-1,1),
 * SW(-1,-1), SE(1,-1)  (PyLB/Streaming.py:28-29).
 *
 * Storage codes (dtype): LBGB_F32 and LBGB_F64 store f itself;
 * LBGB_F16DEV stores the deviation h_i = f_i - w_i scaled by 2^14 as IEEE half
 * (the scale keeps small deviations out of half's subnormal range),
 * LBGB_BF16DEV stores h_i as bfloat16; all arithmetic on those is FP32.
 * LBGB_F32DEV stores h_i as float and collides in deviation form (every
 * rounding is of numbers ~1e-2 instead of ~0.4: about 30x finer than
 * LBGB_F32 at the same 72 bytes per cell and step).
 *
 * The fused solvers (lbgb_step*, lbgb_batch_*) collide every storage but
 * LBGB_F64 in the deviation "pair form": opposite channels enter as
 * a = h_i - h_j and b = h_i + h_j, the momentum is read from the a's, the
 * relaxation of the odd (momentum-carrying) part is written so that the
 * post-collision momentum equals the pre-collision one exactly in exact
 * arithmetic, and the rest population is written last as the node's mass
 * minus the moving channels.  With FP32-rounded lattice weights the direct
 * formula gains a systematic momentum factor (1 + delta) every step; the
 * pair form does not.
 */
#ifndef LBGB_H
#define LBGB_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define LBGB_API __attribute__((visibility("default")))
#else
#define LBGB_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define LBGB_F32 0
#define LBGB_F64 1
#define LBGB_F16DEV 2
#define LBGB_BF16DEV 3
#define LBGB_F32DEV 4

#define LBGB_PERIODIC 0
#define LBGB_CAVITY 1       /* the reference's lid: 6 w rho_lid u0 with its rho_lid, side walls win at the corners */
#define LBGB_CAVITY_LADD 2  /* standard Ladd moving wall, wall density 1, at every lid node (steady-state studies) */

#define LBGB_OK 0
#define LBGB_EINVAL (-1)   /* bad size, pointer or option */
#define LBGB_EDTYPE (-2)   /* unsupported storage code */
#define LBGB_ECUDA (-3)    /* a CUDA call or launch failed */
#define LBGB_EWORKSPACE (-4) /* workspace missing or too small */
#define LBGB_ETIMEOUT (-5) /* a bounded device-side wait gave up */
#define LBGB_EUNSUPPORTED (-6) /* a fused form cannot take these operands: nothing launched, use the unfused calls */

/* Library version as MAJOR*10000 + MINOR*100 + PATCH. */
LBGB_API int lbgb_version(void);

/* Copies the message of the last failure on this host thread into buf
 * (NUL-terminated, truncated to len) and returns its full length. */
LBGB_API int lbgb_last_error(char *buf, size_t len);

/* Equilibrium populations from density and velocity fields (n cells) into
 * f (9 rows, channel stride chan_stride >= n).  dtype: LBGB_F32 or LBGB_F64
 * (rho/ux/uy/f all of that type).
 * Replaces: PyLB.Collision.equilibrium -> d2q9_equilibriumn<T>
 *           (PyLB/Collision.py:21, c/d2q9.h:98-108, c/_lbkernels.cpp:38,45). */
LBGB_API int lbgb_equilibrium(const void *rho, const void *ux, const void *uy, void *f,
                     int64_t n, int64_t chan_stride, int dtype, void *stream);

/* BGK collision in place on f (9 rows of n cells, channel stride chan_stride).
 * Any storage code.  LBGB_F32 and LBGB_F64 compute exactly the operations of
 * the reference's native kernel in its order (every operation rounded on
 * its own, IEEE division, Eigen's fixed-size sum order for rho): the result
 * equals d2q9_colliden<T> bit for bit.  The deviation codes (LBGB_F32DEV and
 * the 16-bit codes) collide in deviation form with the mass-preserving store.
 * Replaces: PyLB.Collision.collide -> d2q9_colliden<T>
 *           (PyLB/Collision.py:21, c/d2q9.h:121-131, c/_lbkernels.cpp:40,47). */
LBGB_API int lbgb_collide(void *f, int64_t n, int64_t chan_stride, int dtype,
                 double omega, void *stream);

/* lbgb_collide with options.  flags = 0: as lbgb_collide.
 * LBGB_COLLIDE_KEEP_MASS: the fused solver's collision instead (the pair
 * form above, on h = f - w for LBGB_F32), whose store writes the rest
 * population last as f_0 + sum_{i>0} (f_i - f_i'), so that each node keeps
 * its mass up to the rounding of that one value (the native float path
 * drifts by ~1e-2 in 500 steps of a 48 x 40 box with resting walls, this
 * one by ~5e-6).  Other bits: LBGB_EINVAL.
 * Same reference interface as lbgb_collide (c/d2q9.h:121-131); the flag has
 * no counterpart there. */
#define LBGB_COLLIDE_KEEP_MASS 1
LBGB_API int lbgb_collide_ex(void *f, int64_t n, int64_t chan_stride, int dtype,
                    double omega, int flags, void *stream);

/* Periodic streaming, pull form, out of place: dst_i(k,l) = src_i(k-cx_i, l-cy_i)
 * with periodic wrap.  src and dst are (9, nx, ny) and must not overlap.
 * Replaces: PyLB.Streaming.stream (PyLB/Streaming.py:33-46). */
LBGB_API int lbgb_stream_periodic(const void *src, void *dst, int nx, int ny, int dtype,
                         void *stream);

/* Streaming with half-way bounce-back on the four walls and a lid at l = ny-1
 * moving with velocity u0 in +x (Ladd correction), out of place; u0 = 0 gives
 * plain bounce-back on all walls.  nx, ny >= 2.
 * Replaces: stream_and_bounce_back(f_ikl, u0)
 *   (simulators/parallel_lid_drive_cavity/cavity_opt1.py:177-245, identical in
 *    cavity_opt0.py:155-223 and cavity_opt2.py:109-177). */
LBGB_API int lbgb_stream_bounce_back(const void *src, void *dst, int nx, int ny,
                            double u0, int dtype, void *stream);

/* The same two streams in place on f (the reference's operators assign the
 * streamed planes back into their argument).  Two launches: the edge values
 * of every 16-row x 512-byte tile that a neighbouring tile pulls are saved
 * into work, then each tile is streamed through shared memory and written
 * back over itself.  Results equal the out-of-place calls bit for bit; about
 * 79 bytes per FP32 cell instead of 144 for out-of-place + copy back.
 * work: a 16-byte aligned device buffer of at least
 * lbgb_stream_inplace_workspace_bytes(nx, ny, dtype) bytes (0 for an invalid
 * grid or storage code): 6 / 16 + 6 element size / 512 elements per cell,
 * 4.7 % of an FP32 lattice (5.2 % FP64); it must not be in use by another call in flight.
 * Replaces: PyLB.Streaming.stream (PyLB/Streaming.py:33-46) and
 *   stream_and_bounce_back(f_ikl, u0) (cavity_opt1.py:177-245), in place. */
LBGB_API size_t lbgb_stream_inplace_workspace_bytes(int nx, int ny, int dtype);
LBGB_API int lbgb_stream_periodic_inplace(void *f, int nx, int ny, int dtype, void *work,
                                 size_t work_bytes, void *stream);
LBGB_API int lbgb_stream_bounce_back_inplace(void *f, int nx, int ny, double u0, int dtype,
                                    void *work, size_t work_bytes, void *stream);

/* One fused time step: pull streaming (boundary = LBGB_PERIODIC or
 * LBGB_CAVITY with lid velocity u0) followed by BGK collision, src -> dst.
 * Any storage code.
 * Replaces the per-step pair stream/stream_and_bounce_back + collide
 *   (cavity_opt2.py:276-277, shear_wave_opt2.py:96-97, cavity_opt1.py:342-343). */
LBGB_API int lbgb_step_fused(const void *src, void *dst, int nx, int ny, int boundary,
                    double omega, double u0, int dtype, void *stream);

/* Copies rows k_begin <= k < k_end of all nine channel planes of a (9, nx, ny)
 * array between any two memories (host or device; the direction comes from
 * the pointers), asynchronously on stream: the transfers of the pipelined
 * host step.  No counterpart in the reference. */
LBGB_API int lbgb_copy_rows(void *dst, const void *src, int nx, int ny, int k_begin, int k_end, int dtype,
                            void *stream);

/* lbgb_step_fused restricted to the rows k_begin <= k < k_end of dst (every
 * row of src may be read): the pieces of a step that is pipelined with the
 * host transfers of neighbouring rows (Lattice.step_host).  Round to nearest
 * for 16-bit storage.  No counterpart in the reference. */
LBGB_API int lbgb_step_fused_rows(const void *src, void *dst, int nx, int ny, int k_begin, int k_end,
                                  int boundary, double omega, double u0, int dtype, void *stream);

/* nsteps fused steps ping-ponging between a and b (a holds the initial
 * state); *which receives 0 if the result is in a, 1 if in b.  Launch-only:
 * suitable for CUDA-graph capture.  Where lbgb_steps_per_launch says 2
 * (LBGB_F32 or LBGB_F32DEV storage, periodic or cavity walls, nx a multiple
 * of 16, ny of 128, 16-byte aligned buffers, LBGB_TUNE_TWO_STEP on and the
 * auto kernel), pairs of steps run as one launch that keeps the intermediate
 * step on chip (k_step2: one read and one write of the lattice per two
 * steps); the results equal single steps bit for bit. */
LBGB_API int lbgb_run_fused(void *a, void *b, int nx, int ny, int boundary,
                   double omega, double u0, int dtype, int nsteps, int *which,
                   void *stream);

/* Steps lbgb_run_fused advances per launch on this lattice (1 or 2; any
 * buffers 16-byte aligned). */
LBGB_API int lbgb_steps_per_launch(int nx, int ny, int boundary, int dtype);

/* As lbgb_run_fused, with stochastic rounding of the 16-bit storage codes
 * (LBGB_F16DEV, LBGB_BF16DEV; other codes run lbgb_run_fused).  Every stored
 * value is rounded up or down at random with the probabilities that make the
 * rounding unbiased, and the rest population keeps each node's mass, so that
 * rounding errors no longer add up step after step in slowly varying flows.
 * The random bits are a hash of (seed, step, cell, channel): results are
 * reproducible.  step_counter: device pointer to one unsigned 64-bit step
 * index, read by every step and advanced by one after it (on the stream), so
 * that graph replays keep drawing fresh bits.  No counterpart in the
 * reference (it has no reduced-precision storage). */
LBGB_API int lbgb_run_fused_sr(void *a, void *b, int nx, int ny, int boundary,
                               double omega, double u0, int dtype, int nsteps,
                               unsigned int seed, unsigned long long *step_counter,
                               int *which, void *stream);

/* Density and velocity of every cell (the diagnostics of cavity_opt2.py:280-281
 * and cavity_opt1.py:154-156).  rho/ux/uy are float for the F32/F16DEV/BF16DEV
 * storage codes and double for F64. */
LBGB_API int lbgb_macroscopic(const void *f, void *rho, void *ux, void *uy, int64_t n,
                     int64_t chan_stride, int dtype, void *stream);

/* Bytes of device workspace lbgb_mass_momentum needs (fixed, small). */
LBGB_API size_t lbgb_mass_momentum_workspace_bytes(void);

/* Total mass and momentum, sum_c sum_i f_i(c) * (1, cx_i, cy_i), accumulated in
 * FP64 with a fixed reduction order (bit-reproducible run to run).  out_dev
 * receives 3 doubles in device memory.  workspace: device buffer of at least
 * lbgb_mass_momentum_workspace_bytes() bytes, 8-byte aligned.
 * Replaces the host-side np.sum(f_ikl) mass checks of the reference drivers. */
LBGB_API int lbgb_mass_momentum(const void *f, int64_t n, int64_t chan_stride, int dtype,
                       double *out_dev, void *workspace, size_t workspace_bytes,
                       void *stream);

/* Allocation-free variant of lbgb_mass_momentum, for callers that may not
 * allocate device memory (a code embedded in an application whose memory
 * manager owns the GPU, or a time loop in which device allocations are
 * forbidden) and therefore cannot pass a workspace.  Same result (FP64 sums;
 * a different but fixed summation order), with the partial sums kept in an
 * array built into the library (1.5 MiB, held on every GPU that loads the
 * library until the process exits).  n must not exceed
 * LBGB_NOALLOC_MAX_CELLS (LBGB_EINVAL otherwise).  The first call on a device
 * looks up the array's device address with that device current; make that
 * first call before any stream capture.  The address is kept for the life of
 * the process: a cudaDeviceReset, or anything else that destroys the
 * device's primary context, invalidates it, so do not call this entry point
 * on a device after such a reset.  All calls share the array: calls
 * whose kernels overlap on the GPU race and must be ordered (one stream, or
 * events).  No counterpart in the reference (it has no GPU path). */
#define LBGB_NOALLOC_MAX_CELLS 268435456LL
LBGB_API int lbgb_mass_momentum_noalloc(const void *f, int64_t n, int64_t chan_stride, int dtype,
                                        double *out_dev, void *stream);

/* Converts populations between storage codes (n cells, channel strides
 * src_stride / dst_stride): e.g. F32 -> F16DEV stores f_i - w_i in half. */
LBGB_API int lbgb_convert(const void *src, int src_dtype, int64_t src_stride, void *dst,
                 int dst_dtype, int64_t dst_stride, int64_t n, void *stream);

/* Batched lattices: many independent (9, nx, ny) lattices of uneven size in
 * one population buffer, advanced by one launch per step over a packed task
 * queue.  One table entry per instance (device memory, 8-byte aligned): */
typedef struct {
    long long offset;        /* element offset of the instance in the buffer */
    int nx, ny;              /* its grid */
    double omega, u0;        /* relaxation parameter, lid velocity (cavity) */
    int vec;                 /* cells per lane: 16/sizeof(element) if its rows hold whole
                                16-byte vectors (and offset is a multiple of it), else 1 */
    unsigned int cell_base;  /* index of its first cell among all instances */
} lbgb_batch_instance;

/* One fused step of every instance, src -> dst (same layout).  tasks: device
 * array of n_tasks int4.  Segment tasks (flat = 0) are {instance, first row,
 * first column, unused}: one warp's work is rows_per_task rows of a
 * 32*vec-cell row segment.  Flat tasks (flat = 1) are {instance, unused,
 * first cell, unused}: lane j takes cells first + 32 r + j of the flattened
 * grid for r < rows_per_task (every lane busy, however short the rows);
 * rows_per_task is then 1, 2, 4 or 8 (LBGB_EINVAL otherwise).
 * total_elems bounds every access (entries that do not fit are skipped).
 * threads: multiple of 32 up to 256; blocks: persistent grid size.
 * Replaces the reference's loop over independent runs of
 * simulators/serial_shear_wave/Python/shear_wave_opt2.py:94-99 (one process
 * per run) with one launch. */
LBGB_API int lbgb_batch_step(const void *src, void *dst, long long total_elems,
                             const void *instances, int n_instances, const void *tasks,
                             long long n_tasks, int rows_per_task, int boundary, int dtype,
                             int threads, int blocks, int flat, void *stream);

/* Per-instance amplitude of the shear mode u_x ~ sin(2 pi l / ny):
 * out_dev[b] = 2/(nx ny) sum_{k,l} u_x(k,l) sin(2 pi l / ny), in FP64.
 * The decay diagnostic of shear_wave_opt1.py:174 / shear_wave_decay.py:155-158. */
LBGB_API int lbgb_batch_shear_amplitude(const void *f, long long total_elems,
                                        const void *instances, int n_instances, int dtype,
                                        double *out_dev, double *partials, void *stream);

/* Scratch of the per-instance diagnostics: partials holds n_instances *
 * LBGB_DIAG_CHUNKS doubles (each instance's cells are reduced in this many
 * chunks in parallel, then combined in chunk order: deterministic). */
#define LBGB_DIAG_CHUNKS 64

/* Steady-state monitor of a batch: out_dev[b] = max over the cells of
 * instance b of |u - u_prev| (x and y components, FP32), then u_prev <- u.
 * u_prev: 2 floats per cell, instances back to back at 2*cell_base.
 * Called every m steps it gives the criterion max|u^(n+m) - u^n| of the
 * steady-cavity data set.  A non-finite velocity (a diverged instance) gives
 * +inf, so it never reads as converged.  No counterpart in the reference. */
LBGB_API int lbgb_batch_velocity_change(const void *f, long long total_elems,
                                        const void *instances, int n_instances, int dtype,
                                        float *u_prev, long long total_cells, float *out_dev,
                                        double *partials, void *stream);

/* Decay diagnostic of the shear-wave scripts: out_dev[0] = 2/ny * max_k
 * |DFT_k(ux[row, :])| (FP64; direct transform over the ny cells of one row,
 * ny <= 4096), ux computed from the populations of the (9, nx, ny) array f.
 * Replaces: simulators/simple_flows/shear_wave_decay.py:155-158 (numpy fft of
 * ux[nx/2, :] on the host every step). */
LBGB_API int lbgb_row_fft_amplitude(const void *f, int nx, int ny, int row, int dtype, double *out_dev,
                                    void *stream);

/* Channel flows with dry wall rows (the simple-flow scripts' convention): the
 * rows y = 0 and y = ny-1 of the (9, nx, ny) array f are walls.  After a push
 * stream, the populations that entered a wall row are reflected into the
 * adjacent fluid row, in place; the top wall moves with uw (SW and SE get
 * -uw/6 and +uw/6).  interior != 0 treats columns 1 .. nx-2 only (the ghost
 * columns of a pressure-periodic channel), clear != 0 zeroes the reflected
 * wall entries afterwards.  dtype LBGB_F32 or LBGB_F64.
 * Replaces: simulators/simple_flows/PoiseuilleFlow.py:59-75 (interior) and
 *           simulators/simple_flows/CouetteFlow.py:106-119 (every column, clear). */
LBGB_API int lbgb_wall_bounce_back(void *f, int nx, int ny, double uw, int interior, int clear, int dtype,
                                   void *stream);

/* Resting solid nodes of any shape, given as a byte mask solid[k * ny + l]
 * (nonzero = solid): after a push stream, every population that entered a
 * solid node returns to the fluid node it came from in the opposite
 * direction (link-wise dry-node bounce-back), in place.  periodic != 0 wraps
 * the neighbours.  For rows of solid nodes this equals the scripts' wall
 * reflection wherever the flow is uniform along the wall; the scripts copy
 * diagonals within the same column (PoiseuilleFlow.py:59-75), the obstacle
 * channel around a rectangle (experimantal_flows/obstacle_canal.py:413-458).
 * dtype LBGB_F32 or LBGB_F64. */
LBGB_API int lbgb_solid_bounce_back(void *f, const void *solid, int nx, int ny, int periodic, int dtype,
                                    void *stream);

/* Pressure-periodic inlet/outlet ghost columns, in place: column 0 becomes
 * f^eq(rho_in, u of column nx-2) + (f - f^eq) of column nx-2, column nx-1
 * becomes f^eq(rho_out, u of column 1) + (f - f^eq) of column 1.
 * Replaces: simulators/simple_flows/PoiseuilleFlow.py:76-88. */
LBGB_API int lbgb_pressure_periodic(void *f, int nx, int ny, double rho_in, double rho_out, int dtype,
                                    void *stream);

/* Start populations for a known flow: equilibrium plus the first-order
 * Chapman-Enskog non-equilibrium part,
 *   f_i = f_i^eq(rho, u) - (3 w_i rho / omega) (c_ia c_ib - delta_ab / 3) d_a u_b,
 * with central-difference velocity gradients (for the cavity boundaries a
 * one-sided quadratic through the wall velocity: 0, or u0 at the lid).
 * post_collision != 0 writes f^eq + (1 - omega) f^neq instead: the state a
 * time step (stream, then collide) leaves, which is what the solvers hold
 * between steps.
 * rho/ux/uy are (nx, ny) fields, f a (9, nx, ny) array, all of type dtype
 * (LBGB_F32 or LBGB_F64).  Used to warm-start the cavity from a predicted
 * flow field; no counterpart in the reference (which starts from rest,
 * simulators/parallel_lid_drive_cavity/cavity_opt1.py:333-335). */
LBGB_API int lbgb_chapman_enskog(const void *rho, const void *ux, const void *uy, void *f, int nx, int ny,
                                 double omega, double u0, int boundary, int post_collision, int dtype,
                                 void *stream);

/* BF16 GEMM with FP32 accumulation: C = alpha * A * B + beta * C for `batch`
 * independent problems.  A (m x k) and B (k x n) are BF16; C is FP32, or BF16
 * when c_bf16 != 0 (rounded once, after the FP32 accumulation).  Element
 * (i, j) of X is X[i * x_rs + j * x_cs] and problem z starts at z * x_bs, so
 * any transposed or strided view works.  engine: 0 tensor cores, choosing
 * the TMA pipeline (cp.async.bulk.tensor operand loads, warp-specialised
 * producer / MMA / epilogue, double-buffered tensor-memory accumulator,
 * persistent CTAs) when B is K-major (b_rs = 1), A is K-major (a_cs = 1) or
 * M-major (a_rs = 1), and their rows are 16-byte aligned, else the
 * staged kernel; 2 the staged tcgen05 kernel only (operands copied into
 * shared memory by the threads); 3 the TMA pipeline only (LBGB_EINVAL for
 * other layouts); 1 CUDA-core reference.  Used by the Fourier-neural-operator
 * surrogate; no counterpart in the reference. */
LBGB_API int lbgb_gemm_bf16(int m, int n, int k, const void *A, long long a_rs, long long a_cs,
                            long long a_bs, const void *B, long long b_rs, long long b_cs,
                            long long b_bs, void *C, long long c_rs, long long c_cs, long long c_bs,
                            int batch, float alpha, float beta, int c_bf16, int engine, void *stream);

/* One problem of lbgb_gemm_bf16 on the TMA pipeline with the surrogate
 * layer's bias and activation in its epilogue: C = alpha A B + beta C, then
 * C += bias[row / rows_per_bias] (bias may be NULL) and, when c_bf16_copy is
 * not NULL, c_bf16_copy = BF16(act ? GELU(C) : C) at the same row and column
 * -- the values of lbgb_gemm_bf16 followed by lbgb_fno_bias_act, without the
 * second pass over C.  A K-major (a_cs = 1), B K-major (element (k, j) at
 * B[j * b_cs + k]), C FP32 row-major with row stride c_rs (column stride 1),
 * C and the copy 16-byte aligned; otherwise LBGB_EUNSUPPORTED (nothing
 * launched).  No counterpart in the reference. */
LBGB_API int lbgb_gemm_bf16_bias_act(int m, int n, int k, const void *A, long long a_rs, long long a_cs,
                                     const void *B, long long b_cs, void *C, long long c_rs, float alpha,
                                     float beta, const float *bias, long long rows_per_bias, int act,
                                     void *c_bf16_copy, void *stream);

/* Synchronizes and reports whether a bounded wait in the tensor-core GEMM gave
 * up since the last reset (LBGB_ETIMEOUT).  No counterpart in the reference. */
LBGB_API int lbgb_gemm_status(int reset);

/* Element-wise and mode-mixing kernels of the Fourier-neural-operator
 * surrogate (activations channel-major: (channels, cols)).  No counterpart in
 * the reference.
 *   to_bf16      y = bf16(x)
 *   bias_act     z += bias[c] (+ extra); v = act(z) (0 identity, 1 GELU), fp32 and/or bf16
 *   gelu_back    dz = dy * GELU'(z) (and its bf16 copy)
 *   row_sum      db[c] = sum_j dy[c, j] (partials: channels * 64 floats of scratch)
 *   mix          per Fourier mode y = sum_c x R (complex, BF16 weights), reading the
 *                transform products P (C, B, 2mk, 2q) and writing the BF16 operand
 *                Ym (O, B, 2q, 2mk) of the inverse transform (q kept ky, mk kept kx)
 *   mix_back     its gradients: dP (BF16) from dYm, and dR (FP32) summed over B
 *   mse          partial sums of (y - t)^2 and d = 2 (y - t) / n
 *   adam         Adam step on FP32 weights, refreshing their BF16 copy
 *   sum_splits   out = beta out + sum of S split-K partial results */
LBGB_API int lbgb_fno_to_bf16(const float *x, void *y, long long n, void *stream);
LBGB_API int lbgb_fno_bias_act(float *z, const float *bias, const float *extra, float *v, void *vb,
                               int channels, long long cols, int act, void *stream);
LBGB_API int lbgb_fno_gelu_back(const float *dy, const float *z, float *dz, void *dzb, long long n,
                                void *stream);
LBGB_API int lbgb_fno_row_sum(const float *dy, float *db, float *partials, int channels, long long cols,
                              void *stream);
LBGB_API int lbgb_fno_mix(const float *P, const void *Rr, const void *Ri, void *Ym, int C, int O, int B,
                          int q, int mk, void *stream);
LBGB_API int lbgb_fno_mix_back(const float *dYm, const float *P, const void *Rr, const void *Ri, void *dP,
                               float *dRr, float *dRi, int C, int O, int B, int q, int mk, void *stream);
LBGB_API int lbgb_fno_mse(const float *y, const float *t, float *d, double *partials, int nparts,
                          long long n, void *stream);
/* lbgb_fno_mse with a weight per plane of `plane` consecutive elements (the
 * (channel, sample) planes of a (C, B, H, W) output): partials of
 * sum w_p (y - t)^2, d = 2 w_p (y - t) / n. */
LBGB_API int lbgb_fno_mse_weighted(const float *y, const float *t, const float *w, long long plane, float *d,
                                   double *partials, int nparts, long long n, void *stream);
LBGB_API int lbgb_fno_adam(float *w, const float *g, float *m, float *v, void *wb, long long n, float lr,
                           float b1, float b2, float eps, int step, float weight_decay, void *stream);
LBGB_API int lbgb_fno_sum_splits(const float *parts, float *out, int S, long long n, float beta,
                                 void *stream);

/* Launch tuning (process-wide; used by the autotuner and the tests).
 *   LBGB_TUNE_KERNEL          0 auto, 1 register kernel, 2 pipelined kernel
 *   LBGB_TUNE_STAGES          shared-memory stages of the pipelined kernel
 *   LBGB_TUNE_WAIT_LIMIT      tries per bounded device-side wait
 *   LBGB_TUNE_PIPE_MIN_CELLS  auto: lattices with fewer cells use the register kernel
 *   LBGB_TUNE_TWO_STEP        1 (default): with the auto kernel, lbgb_run_fused advances
 *                             pairs of steps in one launch (two steps per read and write of
 *                             the lattice) where that kernel applies; 0: one step per launch
 *   LBGB_TUNE_TEST_STALL_PRODUCER  test hook: the pipelined kernel's producer
 *                             delivers nothing, so its consumers' bounded
 *                             waits expire (exercises the timeout path)
 * No counterpart in the reference (it has no GPU path). */
#define LBGB_TUNE_KERNEL 0
#define LBGB_TUNE_STAGES 1
#define LBGB_TUNE_WAIT_LIMIT 2
#define LBGB_TUNE_PIPE_MIN_CELLS 3
#define LBGB_TUNE_TEST_STALL_PRODUCER 4
#define LBGB_TUNE_TWO_STEP 5
LBGB_API int lbgb_set_tuning(int key, long long value);
LBGB_API long long lbgb_get_tuning(int key);

/* Synchronizes the device and reports its status word: LBGB_OK, or
 * LBGB_ETIMEOUT if a bounded wait inside a pipelined kernel gave up since
 * the last reset (reset != 0 clears it).  No counterpart in the reference. */
LBGB_API int lbgb_device_status(int reset);

#ifdef __cplusplus
}
#endif

#endif /* LBGB_H */
