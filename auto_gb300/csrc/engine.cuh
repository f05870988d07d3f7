// Internal declarations shared by the engine's translation units.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lenia_gb300.h"

namespace lenia {

// One kernel's per-step parameters on the device.
struct DevKernel {
    int src, dst;
    float mu, sigma, weight;
};

// One world on the device.  Layouts (HBM):
//   state [C][H][W] float                               channel-major, row-major (reference layout)
//   spec  [C][W/8][H][4] float2   forward half-spectrum, tiles of 4 columns so that a column
//                                 pass reads one contiguous block; column 0 packs the DC column
//                                 (real part) with the Nyquist column W/2 (imaginary part)
//   conv  [K][W/8][H][4] float2   per-kernel convolved spectrum (aliases spec when C = K = 1)
//   khat  [K][W/2+1][HQ] float    real, even kernel spectrum for ky in [0, H/2], times 1/(W*H)
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

// Work items.  Column pass: (world, channel, tile of 4 columns).  Row pass: (world, first of 4 rows).
struct ColItem { int world, chan, tile, pad; };
struct RowItem { int world, row0; };

enum RowMode { MODE_STEP = 0, MODE_FORWARD = 1, MODE_U = 2 };

// Launch shapes a size class can use (threads per CTA); the autotuner picks among them.
constexpr int NT_CHOICES[3] = {128, 256, 512};

// Fused FP32 path (step_fp32.cu).  Return false if the size/thread combination is not built.
bool launch_col_fp32(int H, int nt, int nbuf, const DevWorld* worlds, const ColItem* items, int nitems,
                     const float2* tw, cudaStream_t s);
bool launch_row_fp32(int W, int nt, int mode, int general, const DevWorld* worlds, const RowItem* items,
                     int nitems, int acc_planes, const float2* tw, cudaStream_t s);
size_t col_smem_bytes(int H, int nbuf);
size_t row_smem_bytes(int W, int acc_planes);
int max_smem_optin();
int nt_choice(int n, int which);  // threads per CTA built for transform length n (which = 0 or 1)

// Seeding and statistics (seed.cu).
void launch_seed_patches(float* state, int W, int H, uint32_t seed, const int4* patches, int npatch,
                         cudaStream_t s);
void launch_seed_tiles(float* state, int W, int H, uint32_t seed, const float* pattern, int pw, int ph,
                       int spacing, cudaStream_t s);
void launch_world_stats(const DevWorld* worlds, int nworlds, float* out, cudaStream_t s);

// Tile-layout helpers on the host.
inline size_t spec_elems(int W, int H) { return (size_t)(W / 2) * H; }

}  // namespace lenia
