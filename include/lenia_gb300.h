/*
 * lenia_gb300 -- Lenia-family FFT stepping engine for one NVIDIA GB300 (sm_103a).
 *
 * C ABI of the drop-in for the reference's continuous-CA step.  In the reference
 * (ErikFrankling/auto, Rust + WGSL) an automaton is an `Entry` whose `build(w, h)` returns a
 * `Program` (crates/auto-core/src/automata/mod.rs:14-27, program.rs:102-129) that a `Sim`
 * runs on a `Gpu` (crates/auto-core/src/sim.rs:202-595).  This header replaces that stack for
 * the spectral automata (crates/auto-core/src/automata/spectral.rs): a context owns every
 * device buffer of one or more worlds, and the functions below mirror Sim::new, Sim::step,
 * Sim::write_field / read_field and Sim::tick.
 *
 * Conventions
 *   - Every function returns 0 on success or a negative LENIA_E* code; lenia_last_error()
 *     gives the message (the reference returns Err(String) or panics; nothing here aborts).
 *   - Plain pointers and sizes only.  Host buffers are float32, channel-major then row-major
 *     (c*H*W + y*W + x), the layout of the reference's `state` field.
 *   - One context per host thread; a context uses one CUDA stream on one GPU.
 */
#ifndef LENIA_GB300_H
#define LENIA_GB300_H

#include <stddef.h>
#include <stdint.h>

#if defined(_WIN32)
#define LENIA_API
#else
#define LENIA_API __attribute__((visibility("default")))
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define LENIA_MAX_KERNELS 16
#define LENIA_MAX_CHANNELS 4

/* status codes */
#define LENIA_OK 0
#define LENIA_EINVAL (-1)     /* bad argument: size, index, parameter */
#define LENIA_ESIZE (-2)      /* grid size not supported / world smaller than its kernel */
#define LENIA_ENOMEM (-3)     /* device or host allocation failed */
#define LENIA_ECUDA (-4)      /* a CUDA call failed */
#define LENIA_ENODEV (-5)     /* no usable sm_103 device */
#define LENIA_ESTATE (-6)     /* call not valid in the context's current state */

/* kernel shapes (spectral.rs:288-303, 356-383, 427-433) */
#define LENIA_SHAPE_LENIA 0     /* exp(4 - 1/(q(1-q))) core, q = r/R, with beta shells */
#define LENIA_SHAPE_SL_INNER 1  /* SmoothLife inner disc of radius ra/3, anti-aliased 0.5 */
#define LENIA_SHAPE_SL_OUTER 2  /* SmoothLife outer ring ra/3..ra */
#define LENIA_SHAPE_RING 3      /* MNCA hard ring lo <= r < hi */

/* update rules (spectral.rs:337-345, 396-407, 461-472) */
#define LENIA_RULE_LENIA 0      /* s_d += dt * sum_k w_k * (2 exp(-(U_k-mu_k)^2 / (2 sigma_k^2)) - 1) */
#define LENIA_RULE_SMOOTHLIFE 1 /* Rafler's sigmoid bands on (inner, outer); needs 2 kernels */
#define LENIA_RULE_MNCA 2       /* threshold bands on two neighbourhoods; needs 2 kernels */

/* step implementations */
#define LENIA_PATH_FP32 0       /* fused shared-memory FP32 FFT on the CUDA cores */
#define LENIA_PATH_TF32 1       /* DFT-as-GEMM on tcgen05 tensor cores, TF32 operands */
#define LENIA_PATH_BF16X3 2     /* DFT-as-GEMM on tcgen05, split BF16 (hi*hi + hi*lo + lo*hi) */
#define LENIA_PATH_RADIX2 3     /* the reference's pass structure (radix-2 Stockham, one launch
                                   per stage, spectral.rs:199-264) in FP32 CUDA */

typedef struct LeniaKernel {
    int32_t shape;      /* LENIA_SHAPE_* */
    float radius;       /* R in cells (Lenia), ra (SmoothLife) */
    int32_t nshells;    /* 1..3 beta shells (Lenia) */
    float beta[3];      /* shell peak heights */
    float ring_lo;      /* ring inner radius (MNCA) */
    float ring_hi;      /* ring outer radius (MNCA) */
    int32_t src;        /* source channel */
    int32_t dst;        /* destination channel */
    float mu, sigma;    /* Gaussian growth centre and width (LENIA_RULE_LENIA) */
    float weight;       /* growth weight; weights into one channel should sum to 1 */
} LeniaKernel;

typedef struct LeniaWorldDesc {
    uint32_t width, height;   /* 2^a * 3^b (b <= 1), 32..8192 */
    uint32_t channels;        /* 1..LENIA_MAX_CHANNELS */
    uint32_t nkernels;        /* 1..LENIA_MAX_KERNELS */
    int32_t rule;             /* LENIA_RULE_* */
    float dt;                 /* time step (LENIA_RULE_LENIA) */
    LeniaKernel kernels[LENIA_MAX_KERNELS];
} LeniaWorldDesc;

typedef struct LeniaCtx LeniaCtx;

/* Message for the last failure on this context; with ctx == NULL, the last failure of a
 * call that had no context yet (lenia_create) on this thread.  Never NULL. */
LENIA_API const char* lenia_last_error(const LeniaCtx* ctx);

/* Sim::new (sim.rs:202-282): validate the worlds, allocate every buffer, precompute each
 * kernel spectrum in FP64 on the host (spectral.rs:150-181 does it in f32 on the GPU), zero the
 * states.  `path` is a LENIA_PATH_*.  Sizes the reference would reject with a panic
 * (spectral.rs:103-116) return LENIA_ESIZE. */
LENIA_API int lenia_create(const LeniaWorldDesc* worlds, int32_t nworlds, int32_t path, LeniaCtx** out);
LENIA_API int lenia_destroy(LeniaCtx* ctx);

/* Sim::write_field("state") / read_field("state") (sim.rs:560-595) for one world.
 * count must equal channels*height*width.  Writes are stream-ordered; reads block. */
LENIA_API int lenia_write_state(LeniaCtx* ctx, int32_t world, const float* host, size_t count);
LENIA_API int lenia_read_state(LeniaCtx* ctx, int32_t world, float* host, size_t count);
/* Same with a device pointer on the caller's side (no host staging). */
LENIA_API int lenia_write_state_device(LeniaCtx* ctx, int32_t world, const float* dev, size_t count);
LENIA_API int lenia_read_state_device(LeniaCtx* ctx, int32_t world, float* dev, size_t count);
/* write_field / read_field of every world at once: the states back to back in world order
 * (count = the sum of channels*height*width).  One host<->device copy and, for the read, one
 * synchronisation, where a per-world loop would pay one of each per world.  The reference has
 * one world per Sim, so its nearest equivalent is a loop of write_field / read_field calls. */
LENIA_API int lenia_write_states(LeniaCtx* ctx, const float* host, size_t count);
LENIA_API int lenia_read_states(LeniaCtx* ctx, float* host, size_t count);
/* The same two copies without blocking, for streaming batches of worlds through the engine:
 * the host copies run on two more streams through device staging buffers, so the upload of the
 * next input and the download of the last result overlap the steps in between.  Both are
 * stream-ordered with lenia_step (a write takes effect before the next step; a read returns the
 * states after every step enqueued before it).  The host buffer must stay valid and untouched
 * until lenia_sync returns; page-locked host memory is needed for the copies to overlap.  Fused
 * paths only (LENIA_EINVAL on the radix-2 path). */
LENIA_API int lenia_write_states_async(LeniaCtx* ctx, const float* host, size_t count);
LENIA_API int lenia_read_states_async(LeniaCtx* ctx, float* host, size_t count);

/* Sim::step (sim.rs:297-309): advance every world by `steps`, asynchronously.  Steps are
 * replayed from CUDA graphs of up to 64 steps each. */
LENIA_API int lenia_step(LeniaCtx* ctx, uint32_t steps);
/* lenia_step, then block, and return the device time of those steps in milliseconds from CUDA
 * events recorded on the context's stream around the graph launches. */
LENIA_API int lenia_step_timed(LeniaCtx* ctx, uint32_t steps, float* ms);
/* Gpu::wait (gpu.rs:131-137). */
LENIA_API int lenia_sync(LeniaCtx* ctx);
/* Sim::tick. */
LENIA_API int lenia_tick(const LeniaCtx* ctx, uint64_t* tick);

/* On-device initial states (the reference's init passes, spectral.rs:183-197, 313-335).
 * Tiles: every `spacing` x `spacing` tile whose rand3(tx, ty, seed) is even gets the pw x ph
 * pattern with a quarter turn chosen by (r >> 8) & 3.  Patches: unit_f(rand3(x, y, seed)) in
 * each (x0, y0, w, h) rectangle (torus-wrapped), zero elsewhere.  Channel c of a multichannel
 * world uses seed + c. */
LENIA_API int lenia_seed_tiles(LeniaCtx* ctx, int32_t world, uint32_t seed, const float* pattern, int32_t pw,
                     int32_t ph, int32_t spacing);
LENIA_API int lenia_seed_patches(LeniaCtx* ctx, int32_t world, uint32_t seed, const int32_t* patches_xywh,
                       int32_t npatches);

/* The reference's other seed passes, on the device: SmoothLife's scattered discs of radius 24 in
 * 96-cell tiles (spectral.rs:385-395) and MNCA's random 3x3 blocks with density 0.32
 * (spectral.rs:456-460).  Channel c uses seed + c. */
#define LENIA_SEED_SL_DISCS 1
#define LENIA_SEED_MNCA_BLOCKS 2
LENIA_API int lenia_seed_rule(LeniaCtx* ctx, int32_t world, uint32_t seed, int32_t kind);

/* Headless view (sim.rs:17-41): out_w x out_h RGBA8 pixels of one channel, each the average in
 * light of samples x samples sub-pixel colours at world position origin + (pixel + sub) * scale,
 * black outside the world, with the reference's palettes (spectral.rs:347-349, 410-412, 475-477).
 * No window, swapchain or graphics API: the pixels are written to a host buffer (4*out_w*out_h
 * bytes). */
#define LENIA_PALETTE_LENIA 0
#define LENIA_PALETTE_SMOOTHLIFE 1
#define LENIA_PALETTE_MNCA 2
LENIA_API int lenia_render(LeniaCtx* ctx, int32_t world, int32_t channel, float origin_x, float origin_y, float scale,
                           uint32_t samples, uint32_t out_w, uint32_t out_h, int32_t palette, uint8_t* rgba);

/* Program::cells_per_step (program.rs:116-119) summed over worlds and channels. */
LENIA_API int lenia_cells_per_step(const LeniaCtx* ctx, uint64_t* cells);
/* Program::total_bytes (program.rs:122-129): device bytes this context holds. */
LENIA_API int lenia_memory_bytes(const LeniaCtx* ctx, uint64_t* bytes);

/* Inspection: U_k of the current state (the convolution of kernel k's source channel that the
 * next step will use) as float32 (height x width), and the half-spectrum along x of every row of
 * channel c, which the engine keeps between steps, as complex float32 (height x (width/2+1) x 2).
 * For tests and analysis; they do not advance time. */
LENIA_API int lenia_read_field_u(LeniaCtx* ctx, int32_t world, int32_t kernel, float* host, size_t count);
LENIA_API int lenia_read_spectrum(LeniaCtx* ctx, int32_t world, int32_t channel, float* host, size_t count);

/* Per-world statistics on the device: mass (sum of channel 0) and toroidal centroid (circular
 * mean per axis, in cells).  out: 3 floats per world (mass, cx, cy). */
LENIA_API int lenia_world_stats(LeniaCtx* ctx, float* host_out, size_t count);

/* Autotuner: times the candidate launch shapes of every size class on this context's worlds
 * and keeps the fastest, one dimension after another: the cluster-resident step against the two
 * launches per generation and the persistent step (where they apply), the tensor-core column
 * pass's variants and the
 * tensor-core row pass against the FP32 one (lenia_set_tc_rows, where they apply), then for
 * two-pass classes every pair of column and row launch variants jointly with every chunk budget
 * (worlds per L2-resident run, see lenia_class_shapes) that changes the class's number of chunks,
 * its chunks one after another or on 2 to 4 concurrent lanes (lenia_set_chunk_lanes); then, for
 * the whole step, the split of small classes onto a
 * second graph branch (lenia_set_branch_split).
 * The states are saved first and restored afterwards, also when it fails.  Rebuilds the step
 * graphs.  Optional; defaults are reasonable. */
LENIA_API int lenia_autotune(LeniaCtx* ctx);

/* Pins the launch variant of every size class, in place of the defaults or the autotuner's
 * choice: column 0 and 1 are the scalar build at 64 (80 where its plan has radix 32: columns of 1024,
 * 3072 and 8192) and 128 registers a thread, 2 the paired build (both columns of a tile as f32x2
 * pairs), 3 the scalar build with the radix-16 plan at 64 registers (the same as 0 where the scalar
 * plan has no radix 32); row 0 and 1 the two register caps; -1 keeps a pass's current choice.
 * Results do not depend on the variant beyond float rounding.  Rebuilds the step graphs.  No
 * reference counterpart: the reference has one launch shape per pass. */
LENIA_API int lenia_set_variants(LeniaCtx* ctx, int32_t col_variant, int32_t row_variant);
/* The size classes and their current launch variants: *nclasses = the number of classes; with
 * `out` (count >= 4 * classes) four int32 per class: width, height, column variant, row variant. */
LENIA_API int lenia_class_variants(const LeniaCtx* ctx, int32_t* out, size_t count, size_t* nclasses);
/* The launch shape of every size class, as the autotuner left it: *nclasses = the number of classes;
 * with `out` (count >= 14 * classes) fourteen int32 per class: width, height, column variant, row
 * variant, chunks, worlds, chunk budget in MiB (0: the class is one chunk), rows per row-pass item,
 * 1 if the class runs the cluster-resident step (lenia_set_resident) else 0, that step's launch
 * variant, 1 if its row pass runs on the tensor cores (lenia_set_tc_rows) else 0, the variant of
 * its tensor-core column pass (0: tile groups staged by bulk copies, 1: read after an L2 prefetch,
 * more CTAs an SM; -1: no tensor-core column pass), the launch variant of its persistent step
 * (lenia_set_persistent; -1: the class does not run it), and the lanes its chunks run on
 * (lenia_set_chunk_lanes).
 * A chunk is a run of the class's worlds that the step graph advances through all of its steps
 * before the next run starts, sized so that its states and spectra stay in L2. */
LENIA_API int lenia_class_shapes(const LeniaCtx* ctx, int32_t* out, size_t count, size_t* nclasses);
/* Pins the chunk budget of every size class, in place of the default (32) or the autotuner's
 * choice: a class is split into runs of consecutive worlds of at most `mib` MiB of per-step data each
 * (0: one run per class).  Results do not depend on it (bit for bit); only the L2 traffic does.
 * Rebuilds the step graphs.  No reference counterpart. */
LENIA_API int lenia_set_chunk_budget(LeniaCtx* ctx, uint32_t mib);
/* Pins the lanes of every size class, in place of the default (4) or the autotuner's choice: the
 * chunks of a class on the step graph's main branch run on `lanes` (1..4) concurrent graph branches,
 * chunk c on lane c mod lanes, each lane's chunks one after another, so that the launches of
 * several L2-sized chunks fill the GPU together.  A class of one chunk is unaffected.  Results do
 * not depend on it (bit for bit).  Rebuilds the step graphs.  No reference counterpart. */
LENIA_API int lenia_set_chunk_lanes(LeniaCtx* ctx, int32_t lanes);
/* Branches of the step graph (FP32, TF32 and BF16X3 paths): size classes of at most `cells` cells a world run on graph
 * branches beside the larger classes -- one after another on one side branch (each = 0), or each on
 * a branch of its own (each = 1) -- so that the small classes' latency-bound launches share the GPU
 * with the large classes' (cells = 0: one branch, every class in turn, the default).  lenia_autotune
 * tries every split between class sizes, both ways.  Results do not depend on it (bit for bit).
 * Rebuilds the step graphs.  lenia_branch_split reports the current choice.  No reference
 * counterpart. */
LENIA_API int lenia_set_branch_split(LeniaCtx* ctx, int64_t cells, int32_t each);
LENIA_API int lenia_branch_split(const LeniaCtx* ctx, int64_t* cells, int32_t* each);
/* The cluster-resident step, on (mode 1; 2 + v: on in launch variant v, which transforms 16, 8 or 4
 * sequences at a time for v = 0, 1, 2) or off (mode 0, the default until lenia_autotune chooses)
 * for every size class it applies to: square worlds of 128, 192, 256, 384 or 512 with one channel and one Lenia kernel on
 * the FP32 path.  One launch then advances all of a class's worlds through every generation of a
 * step call, one thread-block cluster (side/32 CTAs) per world with the world's half-spectrum held
 * in the cluster's distributed shared memory, in place of two launches per generation.  The
 * arithmetic is the two-pass step's.  A cluster sync that gives up is reported as LENIA_ECUDA by
 * lenia_sync.  Rebuilds the step graphs.  No reference counterpart (the reference dispatches every
 * pass of every world separately, crates/auto-core/src/sim.rs:297-380). */
LENIA_API int lenia_set_resident(LeniaCtx* ctx, int32_t mode);
/* The persistent step, on (mode 1; 2 + v: on in launch variant v, at most 64 or 128 registers a
 * thread for v = 0, 1) or off (mode 0, the default until lenia_autotune chooses) for every size
 * class it applies to: square worlds of 128, 192, 256, 384, 512, 768, 1024, 2048 or 4096 with one
 * channel and one Lenia kernel on the FP32 path.  One launch then advances all of a class's worlds
 * through every generation of a step call: a grid of resident CTAs claims the two-pass step's column
 * and row items in order, world after world (a world's row items right after the next world's column
 * items, so its half-spectrum is read back from L2), each item waiting, bounded, for the items of the
 * same world it depends on.  The arithmetic is the two-pass step's, bit for bit.  A wait that gives
 * up is reported as LENIA_ECUDA by lenia_sync.  Turning it on turns the cluster-resident step off.
 * Rebuilds the step graphs.  No reference counterpart (the reference dispatches every pass of every
 * world separately, crates/auto-core/src/sim.rs:297-380). */
LENIA_API int lenia_set_persistent(LeniaCtx* ctx, int32_t mode);
/* The tensor-core row pass on (1) or off (0, the default until lenia_autotune chooses per class) on
 * the TF32 and BF16X3 paths: the inverse
 * row DFT, the growth / dt / clamp update and the forward row DFT of the one-channel, one-kernel
 * Lenia step as DFT-as-GEMM on tcgen05 (step rows of 256, 512 and 1024 cells; other classes, and
 * every class when off, take the FP32 row pass).  Rebuilds the step graphs.  No reference
 * counterpart: the reference's row transforms are radix-2 dispatches (spectral.rs:225-264). */
LENIA_API int lenia_set_tc_rows(LeniaCtx* ctx, int32_t on);
/* Pins the variant of every size class's tensor-core column pass (BF16X3, columns of 256..1024), in
 * place of the default (1) or the autotuner's choice: 0 stages each tile group in shared memory by a
 * bulk copy a group ahead; 1 reads it from global memory after an L2 prefetch, which leaves 32 KB of
 * shared memory a CTA free for more CTAs an SM.  Results do not depend on it (bit for bit).  Rebuilds
 * the step graphs.  No reference counterpart. */
LENIA_API int lenia_set_tc_variant(LeniaCtx* ctx, int32_t variant);

/* Host-only (no GPU): the kernel's real, even spectrum as the engine uses it, computed in FP64
 * and rounded to float32, with the inverse-FFT normalisation 1/(width*height) folded in.
 * out[kx * (height/2+1) + ky] for kx in [0, width/2], ky in [0, height/2]; count must be
 * (width/2+1)*(height/2+1).  The reference builds the same spectrum with an f32 FFT of the
 * kernel on the GPU (spectral.rs:150-181). */
LENIA_API int lenia_kernel_spectrum(const LeniaKernel* kernel, uint32_t width, uint32_t height, float* out,
                                    size_t count);

/* Diagnostic: one tensor-core GEMM, D (128 x n) = A (128 x k) * B^T (B is n x k), through the
 * shared-memory operand layouts, descriptors and TMEM reads the tensor-core passes use.
 * A, B, D are row-major float32 on the host; path is LENIA_PATH_TF32 or LENIA_PATH_BF16X3, or
 * LENIA_PATH_BF16X3 | LENIA_SELFTEST_A_MN for A in the MN-major layout of the transposing
 * hand-overs (k <= 64); n in 32..256 (multiple of 32), k in 16..256 (multiple of 16).  No
 * counterpart in the reference (it has no tensor-core code). */
#define LENIA_SELFTEST_A_MN 0x100
LENIA_API int lenia_tc_selftest(int32_t path, int32_t n, int32_t k, const float* a, const float* b, float* d);

/* Failure-detection test hook: every barrier wait in the tensor-core column passes gives up
 * after a bounded number of polls, exits early (after waiting, bounded again, for its own copies
 * and MMAs in flight, and freeing its TMEM) and raises the context's error flag, which
 * lenia_sync / lenia_read_state / lenia_step_timed report as LENIA_ECUDA.  polls_plus_one = 0
 * keeps the default limit of the pass's first wait (the DFT-matrix load); n > 0 sets it to n - 1
 * polls, so 1 makes that wait give up at once, before any MMA is issued.  Takes effect at the next
 * launch (no graph rebuild).  LENIA_ESTATE on a context without a tensor-core path.  The reference
 * surfaces failures as Err(String) rather than panics (crates/auto-core/src/sim.rs:208-219); it has
 * no device-side waits. */
LENIA_API int lenia_tc_set_wait_limit(LeniaCtx* ctx, int32_t polls_plus_one);
/* Failure-detection test hook of the persistent step (lenia_set_persistent): its dependency waits
 * give up after a bounded number of polls (2^22 by default), after which the launch's CTAs stop
 * claiming items and return, and the context's error flag is raised, reported as LENIA_ECUDA by
 * lenia_sync / lenia_read_state.  polls_plus_one = 0 keeps the default; n > 1 sets the limit to n - 1
 * polls; 1 makes every dependency wait give up at once, met or not.  After a give-up the step's
 * results are invalid: rewrite the states (lenia_write_states) before stepping on.  Takes effect at
 * the next launch (no graph rebuild).  The reference has no device-side waits. */
LENIA_API int lenia_persist_set_wait_limit(LeniaCtx* ctx, int32_t polls_plus_one);

/* Steps one world of one channel and one Lenia kernel `steps` times, in place, without allocating
 * device memory.  For callers that cannot call cudaMalloc when they step: an application that
 * has given all device memory to its own pool allocator, or a real-time frame loop where an
 * allocation (which may synchronize the device) would stall the frame.  No counterpart in the
 * reference.
 *   state   device pointer, height*width float32, read and overwritten
 *   khat    device pointer holding lenia_kernel_spectrum()'s output for this kernel and size
 *   stream  a cudaStream_t, or NULL for the default stream; the call is asynchronous on it
 * The scratch it needs (half-spectrum, twiddles, work lists) is a fixed __device__ array of about
 * 4.2 MiB that every GPU loading this library holds until exit, so width*height is limited to
 * 1,048,576 cells (larger returns LENIA_ESIZE).  The first call on a device finds the array's
 * address and fills its twiddle table: make it before any stream capture.  All calls share the
 * array, so calls that overlap on the GPU race; serialise them.  The address is cached per device
 * ordinal, so cudaDeviceReset or a non-primary context between calls is not supported.  A size or
 * launch-configuration error is reported before anything is enqueued; after a launch error (a
 * CUDA error after enqueueing) the state may have been advanced by some of the steps.  Errors:
 * lenia_last_error(NULL). */
LENIA_API int lenia_step_noalloc(float* state, uint32_t width, uint32_t height, const float* khat, float mu,
                                 float sigma, float dt, uint32_t steps, void* stream);

/* ------------------------------------------------------------------------------------------
 * Learned screen proposer: an MLP 16 -> 256 -> 256 -> 3 (ReLU) in BF16 with FP32 accumulation,
 * FP32 master weights and Adam, trained by this library's own forward and backward kernels.
 * Inputs are 16 features of a world's kernel and growth parameters; outputs are
 * P(survives), P(moves), P(explodes) as judged by the simulator.  The reference has no learned
 * component: its world screen samples parameters uniformly (scripts/life_screen.py:143-179).
 * Parameters are one float32 vector: W1 [256x16], b1 [256], W2 [256x256], b2 [256], W3 [3x256],
 * b3 [3] (row-major, output index first). */
typedef struct LeniaMlp LeniaMlp;
LENIA_API int lenia_mlp_create(uint32_t seed, uint32_t max_batch, LeniaMlp** out);
LENIA_API int lenia_mlp_destroy(LeniaMlp* mlp);
LENIA_API int lenia_mlp_param_count(uint32_t* count);
LENIA_API int lenia_mlp_set_params(LeniaMlp* mlp, const float* host, size_t count);
LENIA_API int lenia_mlp_get_params(LeniaMlp* mlp, float* host, size_t count);
/* Gradients of the mean binary cross-entropy over batch x 3 labels (x: batch x 16, y: batch x 3
 * in {0,1}) into grads (param_count floats), without updating the weights. */
LENIA_API int lenia_mlp_gradients(LeniaMlp* mlp, const float* x, const float* y, uint32_t batch, float* grads,
                                  float* loss);
/* One Adam step (beta 0.9 / 0.999) on one batch; returns the batch's mean loss. */
LENIA_API int lenia_mlp_train_step(LeniaMlp* mlp, const float* x, const float* y, uint32_t batch, float lr,
                                   float* loss);
/* Sigmoid outputs for `count` rows of features (count x 3 floats). */
LENIA_API int lenia_mlp_predict(LeniaMlp* mlp, const float* x, uint32_t count, float* probs);

/* Event-timed average device time of the dominant launches of one step, in milliseconds:
 * out[0] = column passes, out[1] = row passes, out[2] = whole step.  Runs `steps` steps. */
LENIA_API int lenia_profile_step(LeniaCtx* ctx, uint32_t steps, float* out3);
/* The same per size class: *nclasses = the number of classes; with `out` (count >= 5 * classes)
 * five floats per class: width, height, column-pass ms and row-pass ms, each the event-timed
 * average over `steps` steps of that class alone (its launches one after another, an event around
 * each, every other class idle), and the ms per step of that class alone as the step graph runs it
 * (a captured graph of `steps` steps: launches back to back, chunks on their lanes).  Advances every
 * class by 3 * `steps`. */
LENIA_API int lenia_profile_classes(LeniaCtx* ctx, uint32_t steps, float* out, size_t count, size_t* nclasses);

#ifdef __cplusplus
}
#endif
#endif /* LENIA_GB300_H */
