// Neural radiance cache: a small MLP evaluated and trained on the tensor
// cores. No counterpart in the reference (a project addition).
//
// Network: 64 inputs -> 4 hidden layers of 64 (ReLU) -> 3 outputs (padded to
// 16), no biases (one input is a constant 1). FP16 weights and activations,
// FP32 accumulation. Inputs (64):
//   [0, 36)   position in the scene box, 6 octaves of sin/cos(2^k pi x) per axis
//   [36, 52)  outgoing direction, real spherical harmonics of degree < 4 (16)
//   [52, 55)  shading normal
//   [55, 58)  albedo
//   58        constant 1 (acts as the first layer's bias)
//   [59, 64)  zero padding
#pragma once
#include <cuda_fp16.h>

#include "common.cuh"

namespace gpugi {
namespace nrc {

constexpr float kPI_F = 3.14159265358979f;
constexpr int kIn = 64, kHidden = 64, kOutPad = 16, kLayers = 5;
// Weight matrix l maps kIn (64) -> kHidden (64) for l < 4 and 64 -> 16 for l = 4.
GPUGI_HD constexpr int out_of(int l) { return l == 4 ? 16 : 64; }
constexpr int kParams = 4 * 64 * 64 + 64 * 16;  // 17,408
// Offset of layer l in a flat parameter array (row-major [in][out]).
GPUGI_HD constexpr int layer_offset(int l) { return l * 64 * 64; }
// Shared-memory row stride (in halves) of the staged weights: 72 = 64 + 8
// keeps the 8 fragment rows of a warp on different banks.
constexpr int kRow = 72;

struct Query {  // one cache lookup / training sample
    float3 pos, dir, normal, albedo;
};

// Frequency + spherical-harmonics encoding of one query into 64 halves.
GPUGI_D void encode(const Query& q, float3 boxMin, float3 boxInvExtent, __half* out) {
    const float p[3] = {(q.pos.x - boxMin.x) * boxInvExtent.x, (q.pos.y - boxMin.y) * boxInvExtent.y,
                        (q.pos.z - boxMin.z) * boxInvExtent.z};
    int k = 0;
    for (int d = 0; d < 3; ++d) {
        float f = kPI_F * p[d];
#pragma unroll
        for (int o = 0; o < 6; ++o) {
            float s, c;
            sincosf(f, &s, &c);
            out[k++] = __float2half(s);
            out[k++] = __float2half(c);
            f *= 2.0f;
        }
    }
    const float x = q.dir.x, y = q.dir.y, z = q.dir.z;
    const float xx = x * x, yy = y * y, zz = z * z;
    const float sh[16] = {0.28209479f,
                          -0.48860251f * y, 0.48860251f * z, -0.48860251f * x,
                          1.09254843f * x * y, -1.09254843f * y * z, 0.31539157f * (3.0f * zz - 1.0f),
                          -1.09254843f * x * z, 0.54627422f * (xx - yy),
                          0.59004359f * y * (-3.0f * xx + yy), 2.89061144f * x * y * z,
                          0.45704580f * y * (1.0f - 5.0f * zz), 0.37317633f * z * (5.0f * zz - 3.0f),
                          0.45704580f * x * (1.0f - 5.0f * zz), 1.44530572f * z * (xx - yy),
                          0.59004359f * x * (-xx + 3.0f * yy)};
#pragma unroll
    for (int i = 0; i < 16; ++i) out[k++] = __float2half(sh[i]);
    out[k++] = __float2half(q.normal.x);
    out[k++] = __float2half(q.normal.y);
    out[k++] = __float2half(q.normal.z);
    out[k++] = __float2half(q.albedo.x);
    out[k++] = __float2half(q.albedo.y);
    out[k++] = __float2half(q.albedo.z);
    out[k++] = __float2half(1.0f);
    while (k < kIn) out[k++] = __float2half(0.0f);
}

}  // namespace nrc
}  // namespace gpugi
