// Buffers of one world on the reference-structured radix-2 path (step_radix2.cu).
#pragma once
#include <cuda_runtime.h>

#include "engine.cuh"

namespace lenia {

struct R2Shape {
    int shape;
    float radius;
    int nshells;
    float beta[3];
    float lo, hi;
};

// Fields of spectral.rs:119-127: state, work (double), spec, kern_i, conv_i.
struct R2World {
    int w, h, k, rule;
    float mu, sigma, dt;
    float* state;
    float2* work[2];
    float2* spec;
    float2* kern[3];
    float* conv[3];
};

int r2_launches_per_step(const R2World& r);
void r2_enqueue_kernel_spectra(R2World& r, const R2Shape* shapes, const float* sums, cudaStream_t s);
void r2_enqueue_convolve(R2World& r, cudaStream_t s);
void r2_enqueue_step(R2World& r, cudaStream_t s);

}  // namespace lenia
