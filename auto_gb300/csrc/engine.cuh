// Internal declarations shared by the engine's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/lenia_gb300.h"

namespace lenia {

// One kernel's per-step parameters on the device.
struct DevKernel {
    int src, dst;
    float mu, sigma, weight;
};

// One world on the device.  Layouts (HBM):
//   state [C][H][W] float                               channel-major, row-major (reference layout)
//   spec  [C][W/(2*TC)][H][TC] float2   half-spectrum along x of every row, in tiles of TC
//                                 columns so that a column pass reads one contiguous block;
//                                 column 0 packs the DC column (real part) with the Nyquist
//                                 column W/2 (imaginary part)
//   conv  [K][W/(2*TC)][H][TC] float2   per-kernel convolved spectrum (aliases spec when C = K = 1)
//   khat  [K][W/2+1][HQ] float    real, even kernel spectrum for ky in [0, H/2], times 1/(W*H);
//                                 HQ = khat_stride(H) >= H/2+1
struct DevWorld {
    int W, H, C, K, rule;
    float dt;
    int HQ;
    float* state;
    float2* spec;
    float2* conv;
    const float* khat;
    float* u_out;  // U_k fields [K][H][W] when a row pass runs in MODE_U
    DevKernel kern[LENIA_MAX_KERNELS];
};

// Spectrum columns per tile: a column pass CTA transforms TC columns of length H.
constexpr int TC = 2;

// Work items.
// A column item: spectrum tile `tile` of channel `chan` with kernel `kernel` (FP32 pass); the
// tensor-core groups use world, chan and the first tile of the group.
struct ColItem { int world, chan, tile, kernel; };
// A row item: rows row0.. of one world.  For Lenia worlds one item per target channel `chan`
// (its kernels, its state update and its forward transform); other rules use chan = 0 and every
// channel.
struct RowItem { int world, row0, chan, pad; };

enum RowMode { MODE_STEP = 0, MODE_FORWARD = 1, MODE_U = 2 };

// Fused FP32 path (step_fp32_*.cu).  Every size is built in two launch variants with the same
// threads per CTA: variant 0 caps registers at 64 per thread (more resident CTAs), variant 1 at
// 128.  The column pass has a third, variant 2: the paired build (both columns of a tile in one
// sequence of f32x2 pairs, half the threads).  The autotuner picks per size class.  The row
// launcher picks its general build from its `general` argument.  Launchers return false if the
// size is not built.
bool launch_col_fp32(int H, int variant, const DevWorld* worlds, const ColItem* items, int nitems,
                     const float2* tw, cudaStream_t s);
bool launch_row_fp32(int W, int variant, int mode, int general, const DevWorld* worlds, const RowItem* items,
                     int nitems, int acc_planes, const float2* tw, cudaStream_t s);
size_t col_smem_bytes(int H);
size_t row_smem_bytes(int W, int acc_planes);
// Column-pass launch variants (launch_col_fp32): 0, 1 scalar builds at two register caps, 2 the paired
// build, 3 the scalar radix-16 build where the scalar plan has radix 32
constexpr int COL_VARIANTS = 4;
// whether the scalar column pass of height H has a radix-16 build beside its radix-32 one (variant 3)
bool col_has_r16_variant(int H);
int row_item_rows(int W, int general);  // rows per row-pass item: 4, or 2 (general step, W >= 2048)
int fp32_local_bytes(int row, int n, int variant);  // spill/stack bytes per thread of a pass instantiation
int max_smem_optin();

// Cluster-resident step (resident.cu): one launch advances every world of a square size class of
// side N (128, 192, 256, 384 or 512; one channel, one Lenia kernel) `gens` generations, one
// thread-block cluster of N/32 CTAs per world.  world_ids: the class's world indices (device).
// err: a device int set to 1 if a cluster sync gave up.  A zero-world call only configures the
// kernel (outside any stream capture).
// Each size is built in RESIDENT_VARIANTS launch variants (sequences per batch, register budget).
constexpr int RESIDENT_VARIANTS = 3;
bool resident_supported(int N);
// co-resident clusters of a variant on this GPU (0: the launch cannot run); configures the kernel
int resident_clusters_that_fit(int N, int variant);
bool launch_resident(int N, int variant, const DevWorld* worlds, const int* world_ids, int nworlds, int gens,
                     const float2* tw, int* err, cudaStream_t s);

// Persistent step (persist.cu): one launch advances every world of a square, one-channel, one-kernel
// Lenia size class of side N through `gens` generations, with the two-pass step's column and row
// items (cols: nc a world, rows: nr a world, world after world) claimed in order by a grid of
// resident CTAs.  ctl: persist_ctl_words(nworlds) ints, zeroed before every launch.  err: two device
// ints, [0] set to 1 if a wait gave up, [1] the waits' poll limit + 1 (0: the default; 1: every
// dependency wait gives up at once, a test hook).  capacity (optional): CTAs the GPU holds at once.
// A zero-world call only configures the kernel (outside any stream capture).
// variant: 0 at most 64 registers a thread, 1 at most 128 (as the two-pass step's launch variants).
constexpr int PERSIST_VARIANTS = 2;
bool persist_supported(int N);
int persist_ctl_words(int nworlds);
bool launch_persist(int N, int variant, const DevWorld* worlds, const ColItem* cols, const RowItem* rows, int nworlds,
                    int ncol, int nrow, int gens, const float2* tw, int* ctl, int* err, cudaStream_t s,
                    int* capacity = nullptr);

// Seeding and statistics (seed.cu).
void launch_seed_patches(float* state, int W, int H, uint32_t seed, const int4* patches, int npatch,
                         cudaStream_t s);
void launch_seed_tiles(float* state, int W, int H, uint32_t seed, const float* pattern, int pw, int ph,
                       int spacing, cudaStream_t s);
void launch_world_stats(const DevWorld* worlds, int nworlds, float* out, cudaStream_t s);
void launch_seed_rule(float* state, int W, int H, uint32_t seed, int kind, cudaStream_t s);
void launch_render(const float* state, int W, int H, float ox, float oy, float scale, int n, int out_w, int out_h,
                   int palette, uchar4* out, cudaStream_t s);

// The message lenia_last_error(NULL) returns on this thread (calls that have no context).
void set_thread_error(const std::string& msg);

// Tile-layout helpers on the host.
inline size_t spec_elems(int W, int H) { return (size_t)(W / 2) * H; }
inline int spec_tiles(int W) { return W / (2 * TC); }
// Row stride of the kernel spectrum (floats): H/2+1 rounded up to a multiple of 4, so that
// every row starts 16-byte aligned and can be moved by a bulk copy.
inline int khat_stride(int H) { return (H / 2 + 1 + 3) / 4 * 4; }

}  // namespace lenia
