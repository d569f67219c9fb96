// Neural radiance cache kernels: fused MLP inference, fused forward +
// backward for training, the weight-gradient GEMM and the Adam step.
//
// Tensor cores via mma.sync m16n8k16 (f16 in, f32 accumulate). A warp owns
// 16 samples at a time; the accumulator fragment of one layer (16 x 8 tiles,
// rows g and g+8, columns 2t and 2t+1 per lane) holds exactly the elements
// the A fragment of the next layer needs, so activations stay in registers
// across all five layers and only the weights come from shared memory.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ctx.cuh"
#include "nrc.cuh"
#include "nrc_tc.cuh"

using namespace gpugi;
using namespace gpugi::nrc;

struct gpugi_nrc {
    gpugi_ctx* ctx = nullptr;
    float3 boxMin, boxInv;
    // Per-sample output gradients are stored in fp16 unnormalised, times
    // lossScale (and clamped below the fp16 range); the 1 / (3 n) of the mean
    // is applied in fp32 after the weight-gradient GEMM.
    float lr = 1e-2f, beta1 = 0.9f, beta2 = 0.99f, eps = 1e-8f, lossScale = 8.0f;
    uint32_t step = 0;
    float* master = nullptr;   // fp32 [l][in][out]
    float* m = nullptr;
    float* v = nullptr;
    float* grad = nullptr;     // fp32 [l][in][out]
    __half* wFwd = nullptr;    // [l][out][in]
    __half* wBwd = nullptr;    // [l][in][out]
    // inference weights: an exponential moving average of the trained weights
    // (decay emaDecay, bias-corrected; the raw weights while emaSteps == 0)
    float* ema = nullptr;      // fp32 running sum (1 - d) sum d^k w
    __half* wInf = nullptr;    // [l][out][in]
    __half* wInfT = nullptr;   // the same, [l][in][out] (tcgen05 inference)
    float emaDecay = 0.99f;
    uint32_t emaSteps = 0;
    __half* acts = nullptr;    // training: X_l per sample, [l][n][64]
    __half* dys = nullptr;     // training: dY_l per sample (scaled), [l][n][64]
    float* lossSum = nullptr;  // device scalar
    uint64_t cap = 0;          // samples the training buffers hold
    // training kernels: tcgen05 (default) or the warp-level mma.sync pair
    uint32_t kernels = GPUGI_NRC_KERNELS_TCGEN05;
    float* partials = nullptr;  // tcgen05 training: weight-gradient sums per CTA [numSMs][kParams]
    // limit of every mbarrier wait of the tcgen05 kernels (a wait that runs
    // out sets GPUGI_DEVERR_WAIT_TIMEOUT and the kernel ends cleanly)
    uint64_t waitNs = 1000000000ull;
    // test support: the tcgen05 kernels issue no MMA and no commit, so
    // their first wait runs out (gpugi_nrc_debug_stall)
    uint32_t stall = 0;
};

namespace gpugi {
namespace nrc {

GPUGI_D void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}
GPUGI_D uint32_t pack2(float lo, float hi) {
    __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}
GPUGI_D float2 unpack2(uint32_t u) {
    __half2 h = *reinterpret_cast<__half2*>(&u);
    return __half22float2(h);
}
// Elements (row, col) and (row + 1, col) of a staged tile (stride kRow) as
// one register: low half = row, high half = row + 1.
GPUGI_D uint32_t pack_pair(const __half* s, int row, int col) {
    __half2 h = __halves2half2(s[row * kRow + col], s[(row + 1) * kRow + col]);
    return *reinterpret_cast<uint32_t*>(&h);
}

// Stage all fp16 weights of one layout into shared memory rows of kRow halves.
// fwd: [l][out][in] (row = out); bwd: [l][in][out] (row = in, out columns).
GPUGI_D void stage_weights(const __half* __restrict__ w, __half* s, bool fwd) {
    for (int l = 0; l < kLayers; ++l) {
        const int rows = fwd ? out_of(l) : kIn, cols = fwd ? kIn : out_of(l);
        const __half* src = w + layer_offset(l);
        __half* dst = s + l * 64 * kRow;
        for (int i = threadIdx.x; i < rows * cols; i += blockDim.x) dst[(i / cols) * kRow + (i % cols)] = src[i];
    }
}

// One layer forward for a warp's 16 rows: acc[j] = A . W (NT n-tiles of 8).
template <int NT>
GPUGI_D void layer_fwd(const uint32_t (&a)[4][4], const __half* sW, float (&acc)[8][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int j = 0; j < NT; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
#pragma unroll
        for (int j = 0; j < NT; ++j) {
            const __half* row = sW + (8 * j + g) * kRow + 16 * kk + 2 * t;
            const uint32_t b0 = *reinterpret_cast<const uint32_t*>(row);
            const uint32_t b1 = *reinterpret_cast<const uint32_t*>(row + 8);
            mma16816(acc[j], a[kk], b0, b1);
        }
    }
}

// Accumulator tiles (n-tiles 2kk, 2kk+1) -> A fragment k-tile kk, with ReLU.
GPUGI_D void acc_to_a(const float (&acc)[8][4], uint32_t (&a)[4][4], bool relu) {
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        float v[8];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            v[i] = acc[2 * kk][i];
            v[4 + i] = acc[2 * kk + 1][i];
        }
        if (relu)
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = fmaxf(v[i], 0.0f);
        a[kk][0] = pack2(v[0], v[1]);
        a[kk][1] = pack2(v[2], v[3]);
        a[kk][2] = pack2(v[4], v[5]);
        a[kk][3] = pack2(v[6], v[7]);
    }
}

// Load a warp's 16 encoded rows (shared, stride kRow) as A fragments.
GPUGI_D void load_a(const __half* sX, uint32_t (&a)[4][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int kk = 0; kk < 4; ++kk) {
        const __half* r0 = sX + g * kRow + 16 * kk + 2 * t;
        const __half* r1 = sX + (g + 8) * kRow + 16 * kk + 2 * t;
        a[kk][0] = *reinterpret_cast<const uint32_t*>(r0);
        a[kk][1] = *reinterpret_cast<const uint32_t*>(r1);
        a[kk][2] = *reinterpret_cast<const uint32_t*>(r0 + 8);
        a[kk][3] = *reinterpret_cast<const uint32_t*>(r1 + 8);
    }
}

GPUGI_D Query load_query(const float* __restrict__ q, uint64_t i) {
    const float* p = q + 12 * i;
    Query r;
    r.pos = make_float3(p[0], p[1], p[2]);
    r.dir = make_float3(p[3], p[4], p[5]);
    r.normal = make_float3(p[6], p[7], p[8]);
    r.albedo = make_float3(p[9], p[10], p[11]);
    return r;
}

// Encode the warp's 16 samples [base, base+16) into shared memory.
GPUGI_D void encode_tile(const float* __restrict__ records, int stride, uint64_t base, uint64_t n, float3 boxMin,
                         float3 boxInv, __half* sX) {
    const int lane = threadIdx.x & 31;
    if (lane < 16) {
        const uint64_t i = base + lane;
        __half row[kIn];
        if (i < n) {
            const float* p = records + (uint64_t)stride * i;
            Query q;
            q.pos = make_float3(p[0], p[1], p[2]);
            q.dir = make_float3(p[3], p[4], p[5]);
            q.normal = make_float3(p[6], p[7], p[8]);
            q.albedo = make_float3(p[9], p[10], p[11]);
            encode(q, boxMin, boxInv, row);
        } else {
            for (int k = 0; k < kIn; ++k) row[k] = __float2half(0.0f);
        }
        for (int k = 0; k < kIn; k += 2)
            *reinterpret_cast<__half2*>(sX + lane * kRow + k) = __halves2half2(row[k], row[k + 1]);
    }
    __syncwarp();
}

// Inference: out[i] = network(query i), 3 floats, clamped at 0.
// With count != NULL the number of queries is min(n, *count) (device side).
__global__ void __launch_bounds__(128) k_nrc_infer(const float* __restrict__ queries, uint64_t n,
                                                   const uint32_t* __restrict__ count,
                                                   const __half* __restrict__ wFwd, float3 boxMin, float3 boxInv,
                                                   float* __restrict__ out) {
    if (count) n = min(n, (uint64_t)*count);
    extern __shared__ __half smem[];
    __half* sW = smem;                                  // 5 x 64 x kRow
    __half* sX = smem + kLayers * 64 * kRow + (threadIdx.x >> 5) * 16 * kRow;
    stage_weights(wFwd, sW, true);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t tile = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile * 16 < n; tile += warps) {
        const uint64_t base = tile * 16;
        encode_tile(queries, 12, base, n, boxMin, boxInv, sX);
        uint32_t a[4][4];
        load_a(sX, a);
        __syncwarp();
        float acc[8][4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            layer_fwd<8>(a, sW + l * 64 * kRow, acc);
            acc_to_a(acc, a, true);
        }
        layer_fwd<2>(a, sW + 4 * 64 * kRow, acc);
        // outputs: n-tile 0 columns 2t, 2t+1 of rows g and g+8; channels 0..2
        if (t < 2) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const uint64_t row = base + g + 8 * h;
                if (row >= n) continue;
#pragma unroll
                for (int c = 0; c < 2; ++c) {
                    const int ch = 2 * t + c;
                    if (ch < 3) out[3 * row + ch] = fmaxf(acc[0][2 * h + c], 0.0f);
                }
            }
        }
    }
}

// Training forward + backward. Samples: 15 floats {query (12), target rgb}.
// Writes every layer's input X_l and scaled output gradient dY_l for the
// weight-gradient GEMM, and accumulates the loss. Relative L2 loss of the
// NRC: (p - y)^2 / (sg(p)^2 + 0.01), averaged over samples and channels.
__global__ void __launch_bounds__(128) k_nrc_fwd_bwd(const float* __restrict__ samples, uint64_t n,
                                                     const uint32_t* __restrict__ count,
                                                     const __half* __restrict__ wFwd, const __half* __restrict__ wBwd,
                                                     float3 boxMin, float3 boxInv, float lossScale,
                                                     __half* __restrict__ acts, __half* __restrict__ dys,
                                                     uint64_t cap, float* lossSum, float* predOut) {
    if (count) n = min(n, (uint64_t)*count);
    extern __shared__ __half smem[];
    __half* sWf = smem;
    __half* sWb = smem + kLayers * 64 * kRow;
    __half* sX = smem + 2 * kLayers * 64 * kRow + (threadIdx.x >> 5) * 16 * kRow;
    stage_weights(wFwd, sWf, true);
    stage_weights(wBwd, sWb, false);
    __syncthreads();
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    const float invCount = n ? 1.0f / (3.0f * (float)n) : 0.0f;
    float lossAcc = 0.0f;
    for (uint64_t tile = (uint64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); tile * 16 < n; tile += warps) {
        const uint64_t base = tile * 16;
        encode_tile(samples, 15, base, n, boxMin, boxInv, sX);
        uint32_t x[kLayers][4][4];  // inputs of every layer (A fragments)
        load_a(sX, x[0]);
        __syncwarp();
        float acc[8][4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            layer_fwd<8>(x[l], sWf + l * 64 * kRow, acc);
            acc_to_a(acc, x[l + 1], true);
        }
        layer_fwd<2>(x[4], sWf + 4 * 64 * kRow, acc);
        // output gradient (scaled), in accumulator layout, n-tiles 0..1
        float dy[8][4];
#pragma unroll
        for (int j = 0; j < 2; ++j)
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int col = 8 * j + 2 * t + (i & 1);
                const uint64_t row = base + g + 8 * (i >> 1);
                float d = 0.0f;
                if (col < 3 && row < n) {
                    const float p = acc[j][i];
                    const float y = samples[15 * row + 12 + col];
                    const float den = p * p + 0.01f;
                    lossAcc += (p - y) * (p - y) / den;
                    d = fminf(fmaxf(2.0f * (p - y) / den * lossScale, -30000.0f), 30000.0f);
                    if (predOut) predOut[3 * row + col] = p;
                }
                dy[j][i] = d;
            }
        // backward through the layers, from the output layer down
#pragma unroll
        for (int l = 4; l >= 0; --l) {
            const int nt = l == 4 ? 2 : 8;  // n-tiles of this layer's output
            // store X_l and dY_l (fp16) for the weight-gradient GEMM
            if (base + 16 <= cap) {
                __half* xo = acts + ((uint64_t)l * cap + base) * 64;
                __half* yo = dys + ((uint64_t)l * cap + base) * 64;
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    *reinterpret_cast<uint32_t*>(xo + g * 64 + 16 * kk + 2 * t) = x[l][kk][0];
                    *reinterpret_cast<uint32_t*>(xo + (g + 8) * 64 + 16 * kk + 2 * t) = x[l][kk][1];
                    *reinterpret_cast<uint32_t*>(xo + g * 64 + 16 * kk + 8 + 2 * t) = x[l][kk][2];
                    *reinterpret_cast<uint32_t*>(xo + (g + 8) * 64 + 16 * kk + 8 + 2 * t) = x[l][kk][3];
                }
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    if (j >= nt) break;
                    *reinterpret_cast<uint32_t*>(yo + g * 64 + 8 * j + 2 * t) = pack2(dy[j][0], dy[j][1]);
                    *reinterpret_cast<uint32_t*>(yo + (g + 8) * 64 + 8 * j + 2 * t) = pack2(dy[j][2], dy[j][3]);
                }
            }
            if (l == 0) break;
            // dX_l = dY_l . W_l^T  (K = out of layer l), then ReLU' of layer l-1's output (= x[l])
            uint32_t ady[4][4];
            const int kt = l == 4 ? 1 : 4;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                if (kk >= kt) break;
                ady[kk][0] = pack2(dy[2 * kk][0], dy[2 * kk][1]);
                ady[kk][1] = pack2(dy[2 * kk][2], dy[2 * kk][3]);
                ady[kk][2] = pack2(dy[2 * kk + 1][0], dy[2 * kk + 1][1]);
                ady[kk][3] = pack2(dy[2 * kk + 1][2], dy[2 * kk + 1][3]);
            }
            float dx[8][4];
#pragma unroll
            for (int j = 0; j < 8; ++j) dx[j][0] = dx[j][1] = dx[j][2] = dx[j][3] = 0.0f;
            const __half* sW = sWb + l * 64 * kRow;  // [in][out]: B[k=out][n=in] = W[in][out]
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                if (kk >= kt) break;
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    const __half* row = sW + (8 * j + g) * kRow + 16 * kk + 2 * t;
                    mma16816(dx[j], ady[kk], *reinterpret_cast<const uint32_t*>(row),
                             *reinterpret_cast<const uint32_t*>(row + 8));
                }
            }
            // ReLU': the activation x[l] (post-ReLU output of layer l-1) holds
            // the same (row, column) positions in this lane.
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const float2 v00 = unpack2(x[l][kk][0]), v10 = unpack2(x[l][kk][1]);
                const float2 v01 = unpack2(x[l][kk][2]), v11 = unpack2(x[l][kk][3]);
                float* d0 = dx[2 * kk];
                float* d1 = dx[2 * kk + 1];
                dy[2 * kk][0] = v00.x > 0.0f ? d0[0] : 0.0f;
                dy[2 * kk][1] = v00.y > 0.0f ? d0[1] : 0.0f;
                dy[2 * kk][2] = v10.x > 0.0f ? d0[2] : 0.0f;
                dy[2 * kk][3] = v10.y > 0.0f ? d0[3] : 0.0f;
                dy[2 * kk + 1][0] = v01.x > 0.0f ? d1[0] : 0.0f;
                dy[2 * kk + 1][1] = v01.y > 0.0f ? d1[1] : 0.0f;
                dy[2 * kk + 1][2] = v11.x > 0.0f ? d1[2] : 0.0f;
                dy[2 * kk + 1][3] = v11.y > 0.0f ? d1[3] : 0.0f;
            }
        }
    }
    for (int off = 16; off > 0; off >>= 1) lossAcc += __shfl_down_sync(0xffffffffu, lossAcc, off);
    if (lane == 0 && lossSum) atomicAdd(lossSum, lossAcc * invCount);
}

// dW_l[in][out] = sum_s X_l[s][in] * dY_l[s][out] over a chunk of samples per
// block; warp w owns rows in [16w, 16w+16). Partial sums go to grad with
// atomics (fp32).
__global__ void __launch_bounds__(128) k_nrc_weight_grad(const __half* __restrict__ acts,
                                                         const __half* __restrict__ dys, uint64_t n,
                                                         const uint32_t* __restrict__ count, uint64_t cap,
                                                         float* __restrict__ grad) {
    if (count) n = min(n, ((uint64_t)*count + 15) / 16 * 16);
    __shared__ __align__(16) __half sX[16 * kRow];
    __shared__ __align__(16) __half sY[16 * kRow];
    const int l = blockIdx.y;
    const int nt = l == 4 ? 2 : 8;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const uint64_t chunk = (n + gridDim.x - 1) / gridDim.x;
    const uint64_t s0 = blockIdx.x * chunk, s1 = min(n, s0 + chunk);
    float acc[8][4];
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
    const __half* X = acts + (uint64_t)l * cap * 64;
    const __half* Y = dys + (uint64_t)l * cap * 64;
    for (uint64_t s = s0; s < s1; s += 16) {
        __syncthreads();
        for (int i = threadIdx.x; i < 16 * 32; i += blockDim.x) {  // 16 rows x 32 half2
            const int r = i >> 5, c = (i & 31) * 2;
            const uint64_t row = s + r;
            __half2 xv = __floats2half2_rn(0.0f, 0.0f), yv = xv;
            if (row < s1) {
                xv = *reinterpret_cast<const __half2*>(X + row * 64 + c);
                yv = *reinterpret_cast<const __half2*>(Y + row * 64 + c);
            }
            *reinterpret_cast<__half2*>(sX + r * kRow + c) = xv;
            *reinterpret_cast<__half2*>(sY + r * kRow + c) = yv;
        }
        __syncthreads();
        // A[m=in][k=sample] = X[k][m]; B[k=sample][n=out] = Y[k][n]: both are
        // column reads of the staged rows, packed two halves per register.
        const int m = 16 * warp + g;
        uint32_t a[4];
        a[0] = pack_pair(sX, 2 * t, m);
        a[1] = pack_pair(sX, 2 * t, m + 8);
        a[2] = pack_pair(sX, 2 * t + 8, m);
        a[3] = pack_pair(sX, 2 * t + 8, m + 8);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            if (j >= nt) break;
            const int col = 8 * j + g;
            mma16816(acc[j], a, pack_pair(sY, 2 * t, col), pack_pair(sY, 2 * t + 8, col));
        }
    }
    float* G = grad + layer_offset(l);
    const int outs = out_of(l);
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        if (j >= nt) break;
        const int r0 = 16 * warp + g, c0 = 8 * j + 2 * t;
        atomicAdd(G + r0 * outs + c0, acc[j][0]);
        atomicAdd(G + r0 * outs + c0 + 1, acc[j][1]);
        atomicAdd(G + (r0 + 8) * outs + c0, acc[j][2]);
        atomicAdd(G + (r0 + 8) * outs + c0 + 1, acc[j][3]);
    }
}

// Adam (fp32 master weights), then the two fp16 layouts.
// With count != NULL the gradient is the sum over min(*count, cap) samples
// and gradScale is 1 / (3 count lossScale); no samples: no update.
__global__ void k_nrc_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ grad, float gradScale, const uint32_t* __restrict__ count,
                           uint64_t cap, float lossScale, float lr, float b1, float b2, float eps, float c1, float c2,
                           __half* __restrict__ wFwd, __half* __restrict__ wBwd, float* __restrict__ ema,
                           float emaDecay, float emaCorr, __half* __restrict__ wInf, __half* __restrict__ wInfT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    bool update = true;
    if (count) {
        const uint64_t c = min((uint64_t)*count, cap);
        update = c > 0;
        gradScale = update ? 1.0f / (3.0f * (float)c * lossScale) : 0.0f;
    }
    const float gr = grad[i] * gradScale;
    if (update && isfinite(gr)) {
        const float mi = b1 * m[i] + (1.0f - b1) * gr;
        const float vi = b2 * v[i] + (1.0f - b2) * gr * gr;
        m[i] = mi;
        v[i] = vi;
        w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
    const int l = i < 4 * 4096 ? i / 4096 : 4;
    const int local = i - layer_offset(l), outs = out_of(l);
    const int in = local / outs, out = local % outs;
    const __half h = __float2half(w[i]);
    wBwd[i] = h;
    wFwd[layer_offset(l) + out * kIn + in] = h;
    float inf = w[i];
    if (emaDecay > 0.0f) {
        const float e = emaDecay * ema[i] + (1.0f - emaDecay) * w[i];
        ema[i] = e;
        inf = e * emaCorr;
    }
    wInf[layer_offset(l) + out * kIn + in] = __float2half(inf);
    wInfT[i] = __float2half(inf);
}

// fp16 layouts of the master weights (after creation or set_weights); the
// inference weights restart from them.
__global__ void k_nrc_publish(const float* __restrict__ w, __half* __restrict__ wFwd, __half* __restrict__ wBwd,
                              float* __restrict__ ema, __half* __restrict__ wInf, __half* __restrict__ wInfT) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    const int l = i < 4 * 4096 ? i / 4096 : 4;
    const int local = i - layer_offset(l), outs = out_of(l);
    const int in = local / outs, out = local % outs;
    const __half h = __float2half(w[i]);
    wBwd[i] = h;
    wFwd[layer_offset(l) + out * kIn + in] = h;
    wInf[layer_offset(l) + out * kIn + in] = h;
    wInfT[i] = h;
    ema[i] = 0.0f;
}

// The input encoding alone (64 halves per query), for inspection and tests.
__global__ void k_nrc_encode(const float* __restrict__ queries, uint64_t n, float3 boxMin, float3 boxInv,
                             __half* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    __half row[kIn];
    encode(load_query(queries, i), boxMin, boxInv, row);
    for (int k = 0; k < kIn; ++k) out[i * kIn + k] = row[k];
}

// ------------------------------------------------ tcgen05 training kernel
// One CTA per SM runs 128-sample tiles: thread t owns sample t of a tile
// (TMEM lane t). Per tile, ten MMA phases, each issued by thread 0 and
// completed through one mbarrier: forward layers 0-4 (D = X_l W_l), backward
// layers 4-1 (D = dY_l W_l^T), then the weight gradients of the tile,
// accumulated in TMEM across all tiles of the CTA. Between phases the
// threads read D from TMEM, apply ReLU (forward) or the ReLU derivative
// (backward), and write the next operand to shared memory as fp16.
// Shared memory (core-matrix layouts, see nrc_tc.cuh):
//   W   the five weight matrices as stored, [in][out] with out contiguous:
//       the forward B (K = in, MN-major) and, through a K-major descriptor of
//       the same bytes, the backward B = W^T (K = out).
//   X   inputs of all layers of the tile, 320 features per sample
//       (X_l = features [64 l, 64 l + 64)), sample groups of 8 rows 5120 B
//       apart: the forward A (K-major) and, MN-major, the A of the weight
//       gradient of a layer pair: [X_l^T ; X_{l+1}^T] is M = 128.
//   Y   output gradients of all layers (dY_l = features [64 l, 64 l +
//       out_l), 272 features): the backward A and the weight-gradient B
//       [dY_l | dY_{l+1}] (N = 128).
// The weight gradient of a pair is the diagonal blocks of the 128 x 128
// product: rows 0-63 x columns 0-63 = dW_l, rows 64-127 x columns 64-127 =
// dW_{l+1}; layer 4 alone uses N = 16 (rows 64-127 of its D are unused).
// TMEM (512 columns): D of a phase at column 0, weight gradients of pairs
// (0,1), (2,3) and layer 4 at columns 128, 256 and 384. Each CTA writes its
// weight-gradient sums to its own row of `partials`.
namespace tcl {
constexpr uint32_t kXSG = 40 * 128, kYSG = 34 * 128;
constexpr uint32_t kWOff = 0, kWBytes = 4 * 8192 + 2048;
constexpr uint32_t kXOff = kWBytes, kXBytes = 16 * kXSG;
constexpr uint32_t kYOff = kXOff + kXBytes + 2048;  // 2 KB pad: rows 64-127 of layer 4's X^T read past X
constexpr uint32_t kYBytes = 16 * kYSG;
constexpr uint32_t kSmem = kYOff + kYBytes + 1024;  // + alignment slack
constexpr uint32_t kColD = 0;
GPUGI_HD constexpr uint32_t col_w(int pair) { return 128u * (uint32_t)(pair + 1); }  // 128, 256, 384
GPUGI_HD constexpr uint32_t w_off(int l) { return kWOff + (uint32_t)l * 8192; }
GPUGI_HD constexpr uint32_t w_kstride(int l) { return (uint32_t)out_of(l) / 8 * 128; }  // between 8-row groups of in
}  // namespace tcl

GPUGI_D uint4 pack8(const float* v, bool relu) {
    uint32_t u[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float a = relu ? fmaxf(v[2 * i], 0.0f) : v[2 * i], b = relu ? fmaxf(v[2 * i + 1], 0.0f) : v[2 * i + 1];
        u[i] = pack2(a, b);
    }
    return make_uint4(u[0], u[1], u[2], u[3]);
}

__global__ void __launch_bounds__(128, 1) k_nrc_train_tc(const float* __restrict__ samples, uint64_t n,
                                                         const uint32_t* __restrict__ count,
                                                         const __half* __restrict__ wBwd, float3 boxMin,
                                                         float3 boxInv, float lossScale, float* __restrict__ partials,
                                                         float* lossSum, float* predOut, uint32_t* errWord,
                                                         uint64_t waitNs, uint32_t stall) {
    using namespace tc;
    using namespace tcl;
    if (count) n = min(n, (uint64_t)*count);
    extern __shared__ uint8_t smemRaw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smemRaw) + 1023) & ~uintptr_t(1023));
    __shared__ uint64_t bar;
    __shared__ uint32_t tmemBase;
    __shared__ float lossWarp[4];
    const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
    // weights, 16-byte chunks of 8 consecutive outputs
    for (int l = 0; l < kLayers; ++l) {
        const int outs = out_of(l), chunks = 64 * outs / 8;
        const uint4* src = reinterpret_cast<const uint4*>(wBwd + layer_offset(l));
        for (int c = t; c < chunks; c += blockDim.x) {
            const int in = c / (outs / 8), o8 = c % (outs / 8);
            *reinterpret_cast<uint4*>(sm + w_off(l) + cm_off(in, 8 * o8, w_kstride(l), 128)) = src[c];
        }
    }
    if (t == 0) bar_init(&bar, 1);
    if (warp == 0) tmem_alloc(&tmemBase, 512);
    fence_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tm = tmemBase;
    const uint32_t lanes = (uint32_t)(32 * warp) << 16;
    const uint32_t xs = smem_addr(sm + kXOff), ys = smem_addr(sm + kYOff), ws = smem_addr(sm + kWOff);
    uint8_t* xRow = sm + kXOff + (t / 8) * kXSG + (t % 8) * 16;  // + feature group x 128
    uint8_t* yRow = sm + kYOff + (t / 8) * kYSG + (t % 8) * 16;
    uint32_t parity = 0;
    bool any = false, failed = false;
    float lossAcc = 0.0f;
    const float invCount = n ? 1.0f / (3.0f * (float)n) : 0.0f;
    const uint64_t tiles = (n + 127) / 128;
    // one MMA phase: thread 0 issues, everyone waits; false on a timeout
    auto phase_wait = [&]() {
        const bool ok = bar_wait(&bar, parity, waitNs);
        parity ^= 1u;
        fence_after();
        return ok;
    };
    for (uint64_t tile = blockIdx.x; tile < tiles && !failed; tile += gridDim.x) {
        const uint64_t row = tile * 128 + (uint64_t)t;
        const bool live = row < n;
        __align__(16) __half enc[kIn];
        float y[3] = {0.0f, 0.0f, 0.0f};
        if (live) {
            const float* p = samples + 15 * row;
            Query q;
            q.pos = make_float3(p[0], p[1], p[2]);
            q.dir = make_float3(p[3], p[4], p[5]);
            q.normal = make_float3(p[6], p[7], p[8]);
            q.albedo = make_float3(p[9], p[10], p[11]);
            encode(q, boxMin, boxInv, enc);
            y[0] = p[12];
            y[1] = p[13];
            y[2] = p[14];
        } else {
#pragma unroll
            for (int k = 0; k < kIn; ++k) enc[k] = __float2half(0.0f);
        }
        // the previous tile's weight-gradient MMAs read X and Y until here
        if (any) failed = !phase_wait();
#pragma unroll
        for (int j = 0; j < 8; ++j) *reinterpret_cast<uint4*>(xRow + j * 128) = *reinterpret_cast<const uint4*>(enc + 8 * j);
        fence_smem();
        fence_before();
        if (__syncthreads_or(failed)) break;
        fence_after();
        any = true;
        // forward
        for (int l = 0; l < kLayers && !failed; ++l) {
            const int outs = out_of(l);
            if (t == 0 && !stall) {
                const uint32_t id = idesc(128, outs, false, true);
                for (int s = 0; s < 4; ++s)
                    mma(tm + kColD, desc(xs + l * 1024 + s * 256, 128, kXSG),
                        desc(ws + w_off(l) + s * 2 * w_kstride(l), w_kstride(l), 128), id, s > 0);
                commit(&bar);
            }
            failed = !phase_wait();
            if (l < 4) {
                uint32_t r[4][16];
#pragma unroll
                for (int c = 0; c < 4; ++c) ld16(tm + lanes + kColD + 16 * c, r[c]);
                ld_wait();
#pragma unroll
                for (int c = 0; c < 4; ++c)
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        float v[8];
#pragma unroll
                        for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[c][8 * h + i]);
                        *reinterpret_cast<uint4*>(xRow + (8 * (l + 1) + 2 * c + h) * 128) = pack8(v, true);
                    }
            } else {
                uint32_t r[16];
                ld16(tm + lanes + kColD, r);
                ld_wait();
                float d[16];
#pragma unroll
                for (int c = 0; c < 16; ++c) d[c] = 0.0f;
                if (live) {
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const float pr = __uint_as_float(r[c]);
                        const float den = pr * pr + 0.01f;
                        lossAcc += (pr - y[c]) * (pr - y[c]) / den;
                        d[c] = fminf(fmaxf(2.0f * (pr - y[c]) / den * lossScale, -30000.0f), 30000.0f);
                        if (predOut) predOut[3 * row + c] = pr;
                    }
                }
                *reinterpret_cast<uint4*>(yRow + 32 * 128) = pack8(d, false);
                *reinterpret_cast<uint4*>(yRow + 33 * 128) = pack8(d + 8, false);
            }
            fence_smem();
            fence_before();
            failed = __syncthreads_or(failed);
            fence_after();
        }
        // backward: dY_{l-1} = (dY_l W_l^T) * [X_l > 0]
        for (int l = 4; l >= 1 && !failed; --l) {
            if (t == 0 && !stall) {
                const uint32_t id = idesc(128, 64, false, false);
                const int steps = l == 4 ? 1 : 4;
                for (int s = 0; s < steps; ++s)
                    mma(tm + kColD, desc(ys + l * 1024 + s * 256, 128, kYSG),
                        desc(ws + w_off(l) + s * 256, 128, w_kstride(l)), id, s > 0);
                commit(&bar);
            }
            failed = !phase_wait();
            uint32_t r[4][16];
#pragma unroll
            for (int c = 0; c < 4; ++c) ld16(tm + lanes + kColD + 16 * c, r[c]);
            ld_wait();
#pragma unroll
            for (int c = 0; c < 4; ++c)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const uint4 xa = *reinterpret_cast<const uint4*>(xRow + (8 * l + 2 * c + h) * 128);
                    const uint32_t xw[4] = {xa.x, xa.y, xa.z, xa.w};
                    float v[8];
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        const float2 xv = unpack2(xw[i]);
                        v[2 * i] = xv.x > 0.0f ? __uint_as_float(r[c][8 * h + 2 * i]) : 0.0f;
                        v[2 * i + 1] = xv.y > 0.0f ? __uint_as_float(r[c][8 * h + 2 * i + 1]) : 0.0f;
                    }
                    *reinterpret_cast<uint4*>(yRow + (8 * (l - 1) + 2 * c + h) * 128) = pack8(v, false);
                }
            fence_smem();
            fence_before();
            failed = __syncthreads_or(failed);
            fence_after();
        }
        if (failed) break;
        // weight gradients of the tile, accumulated over the CTA's tiles;
        // completion is awaited before the next tile overwrites X and Y
        if (t == 0 && !stall) {
            const bool first = tile == blockIdx.x;
            for (int pr = 0; pr < 3; ++pr) {
                const uint32_t id = idesc(128, pr < 2 ? 128 : 16, true, true);
                for (int s = 0; s < 8; ++s)
                    mma(tm + col_w(pr), desc(xs + 2 * pr * 1024 + s * 2 * kXSG, kXSG, 128),
                        desc(ys + 2 * pr * 1024 + s * 2 * kYSG, kYSG, 128), id, !(first && s == 0));
            }
            commit(&bar);
        }
    }
    if (any && !failed) failed = !phase_wait();
    failed = __syncthreads_or(failed);
    // this CTA's weight-gradient sums (zero when it had no tile)
    float* P = partials + (size_t)blockIdx.x * kParams;
    if (!failed && any) {
        for (int pr = 0; pr < 2; ++pr) {
            const int l = 2 * pr + (t >= 64 ? 1 : 0), in = t & 63;
            const uint32_t col0 = col_w(pr) + (t >= 64 ? 64 : 0);
            uint32_t r[4][16];
#pragma unroll
            for (int c = 0; c < 4; ++c) ld16(tm + lanes + col0 + 16 * c, r[c]);
            ld_wait();
            float* G = P + layer_offset(l) + in * 64;
#pragma unroll
            for (int c = 0; c < 4; ++c)
#pragma unroll
                for (int i = 0; i < 16; i += 4)
                    *reinterpret_cast<float4*>(G + 16 * c + i) =
                        make_float4(__uint_as_float(r[c][i]), __uint_as_float(r[c][i + 1]),
                                    __uint_as_float(r[c][i + 2]), __uint_as_float(r[c][i + 3]));
        }
        if (t < 64) {
            uint32_t r[16];
            ld16(tm + lanes + col_w(2), r);
            ld_wait();
            float* G = P + layer_offset(4) + t * 16;
#pragma unroll
            for (int i = 0; i < 16; i += 4)
                *reinterpret_cast<float4*>(G + i) = make_float4(__uint_as_float(r[i]), __uint_as_float(r[i + 1]),
                                                                __uint_as_float(r[i + 2]), __uint_as_float(r[i + 3]));
        } else {
            uint32_t r[16];
            ld16(tm + lanes + col_w(2), r);  // the warp-wide load of the unused rows 64-127
            ld_wait();
        }
    } else {
        for (int i = t; i < kParams; i += blockDim.x) P[i] = 0.0f;
    }
    if (failed && t == 0) atomicOr(errWord, GPUGI_DEVERR_WAIT_TIMEOUT);
    for (int off = 16; off > 0; off >>= 1) lossAcc += __shfl_down_sync(0xffffffffu, lossAcc, off);
    if (lane == 0) lossWarp[warp] = lossAcc;
    fence_before();
    __syncthreads();
    fence_after();
    if (t == 0 && lossSum) atomicAdd(lossSum, (lossWarp[0] + lossWarp[1] + lossWarp[2] + lossWarp[3]) * invCount);
    if (warp == 0) tmem_free(tm, 512);
}

// ----------------------------------------------- tcgen05 inference kernel
// Two warpgroups per CTA, each running its own chain of 128-query tiles:
// thread t of a warpgroup owns query t of the tile (TMEM lane t), one
// thread per warpgroup issues the five layers' MMAs (D = X W_l) into the
// warpgroup's 64 TMEM columns and its mbarrier tracks them; between layers
// the warpgroup turns D into the next layer's fp16 input (ReLU) in its own
// 16 KB X buffer. The weights (the moving average, [in][out] as the
// training weights) are staged once per CTA. 3 CTAs fit an SM (66 KB of
// shared memory, 128 TMEM columns each), so six chains overlap their
// latencies.
namespace tci {
constexpr uint32_t kXSG = 8 * 128, kXBytes = 16 * kXSG;
constexpr uint32_t kWBytes = tcl::kWBytes;
constexpr uint32_t kSmem = kWBytes + 2 * kXBytes + 1024;
}  // namespace tci

// A barrier of the warpgroup's 128 threads that also ORs a flag over them.
GPUGI_D bool wg_any(int wg, bool v) {
    uint32_t r;
    if (wg == 0)
        asm volatile("{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.or.pred p, 1, 128, q;\nselp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(r)
                     : "r"((uint32_t)v)
                     : "memory");
    else
        asm volatile("{\n.reg .pred p, q;\nsetp.ne.u32 q, %1, 0;\nbar.red.or.pred p, 2, 128, q;\nselp.u32 %0, 1, 0, p;\n}\n"
                     : "=r"(r)
                     : "r"((uint32_t)v)
                     : "memory");
    return r != 0;
}

__global__ void __launch_bounds__(256) k_nrc_infer_tc(const float* __restrict__ queries, uint64_t n,
                                                      const uint32_t* __restrict__ count,
                                                      const __half* __restrict__ wInfT, float3 boxMin, float3 boxInv,
                                                      float* __restrict__ out, uint32_t* errWord, uint64_t waitNs,
                                                      uint32_t stall) {
    using namespace tc;
    using namespace tcl;
    if (count) n = min(n, (uint64_t)*count);
    extern __shared__ uint8_t smemRaw[];
    uint8_t* sm = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smemRaw) + 1023) & ~uintptr_t(1023));
    __shared__ uint64_t bars[2];
    __shared__ uint32_t tmemBase;
    const int t = threadIdx.x, wg = t >> 7, lt = t & 127, warp = t >> 5;
    for (int l = 0; l < kLayers; ++l) {
        const int outs = out_of(l), chunks = 64 * outs / 8;
        const uint4* src = reinterpret_cast<const uint4*>(wInfT + layer_offset(l));
        for (int c = t; c < chunks; c += blockDim.x) {
            const int in = c / (outs / 8), o8 = c % (outs / 8);
            *reinterpret_cast<uint4*>(sm + w_off(l) + cm_off(in, 8 * o8, w_kstride(l), 128)) = src[c];
        }
    }
    if (t == 0) {
        bar_init(&bars[0], 1);
        bar_init(&bars[1], 1);
    }
    if (warp == 0) tmem_alloc(&tmemBase, 128);
    fence_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tm = tmemBase + 64u * (uint32_t)wg;
    const uint32_t lanes = (uint32_t)(32 * (warp & 3)) << 16;
    uint8_t* xb = sm + tci::kWBytes + (uint32_t)wg * tci::kXBytes;
    const uint32_t xs = smem_addr(xb), ws = smem_addr(sm);
    uint8_t* xRow = xb + (lt / 8) * tci::kXSG + (lt % 8) * 16;
    uint64_t* bar = &bars[wg];
    uint32_t parity = 0;
    bool failed = false;
    const uint64_t tiles = (n + 127) / 128;
    for (uint64_t tile = 2 * (uint64_t)blockIdx.x + wg; tile < tiles && !failed; tile += 2 * (uint64_t)gridDim.x) {
        const uint64_t row = tile * 128 + (uint64_t)lt;
        {
            __align__(16) __half enc[kIn];
            if (row < n) {
                const float* p = queries + 12 * row;
                Query q;
                q.pos = make_float3(p[0], p[1], p[2]);
                q.dir = make_float3(p[3], p[4], p[5]);
                q.normal = make_float3(p[6], p[7], p[8]);
                q.albedo = make_float3(p[9], p[10], p[11]);
                encode(q, boxMin, boxInv, enc);
            } else {
#pragma unroll
                for (int k = 0; k < kIn; ++k) enc[k] = __float2half(0.0f);
            }
#pragma unroll
            for (int j = 0; j < 8; ++j)
                *reinterpret_cast<uint4*>(xRow + j * 128) = *reinterpret_cast<const uint4*>(enc + 8 * j);
        }
        for (int l = 0; l < kLayers; ++l) {
            // the layer's barrier also agrees on a timeout: a warpgroup
            // leaves together, never with some threads waiting here
            fence_smem();
            fence_before();
            failed = wg_any(wg, failed);
            fence_after();
            if (failed) break;
            const int outs = out_of(l);
            if (lt == 0 && !stall) {
                const uint32_t id = idesc(128, outs, false, true);
                for (int s = 0; s < 4; ++s)
                    mma(tm, desc(xs + s * 256, 128, tci::kXSG),
                        desc(ws + w_off(l) + s * 2 * w_kstride(l), w_kstride(l), 128), id, s > 0);
                commit(bar);
            }
            if (!bar_wait(bar, parity, waitNs)) failed = true;
            parity ^= 1u;
            fence_after();
            if (failed) continue;  // on to the next layer's barrier, which ends the tile
            if (l < 4) {
                // the MMA has read X: overwrite it with this layer's output
#pragma unroll
                for (int c = 0; c < 4; ++c) {
                    uint32_t r[16];
                    ld16(tm + lanes + 16 * c, r);
                    ld_wait();
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        float v[8];
#pragma unroll
                        for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[8 * h + i]);
                        *reinterpret_cast<uint4*>(xRow + (2 * c + h) * 128) = pack8(v, true);
                    }
                }
            } else {
                uint32_t r[16];
                ld16(tm + lanes, r);
                ld_wait();
                if (row < n)
#pragma unroll
                    for (int c = 0; c < 3; ++c) out[3 * row + c] = fmaxf(__uint_as_float(r[c]), 0.0f);
            }
        }
        failed = wg_any(wg, failed);  // the warpgroup takes its next tile, or leaves, together
    }
    if (failed && lt == 0) atomicOr(errWord, GPUGI_DEVERR_WAIT_TIMEOUT);
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) tmem_free(tmemBase, 128);
}

// grad[i] = sum over the CTAs' partial sums, in a fixed order
// (deterministic): a block of 256 threads sums 64 parameters, four row
// groups of it in parallel, then the four group sums in order.
__global__ void __launch_bounds__(256) k_nrc_sum_partials(const float* __restrict__ partials, int rows,
                                                          float* __restrict__ grad) {
    __shared__ float part[4][64];
    const int c = threadIdx.x & 63, g = threadIdx.x >> 6;
    const int i = blockIdx.x * 64 + c;
    float s = 0.0f;
    if (i < kParams)
        for (int r = g; r < rows; r += 4) s += partials[(size_t)r * kParams + i];
    part[g][c] = s;
    __syncthreads();
    if (g == 0 && i < kParams) grad[i] = ((part[0][c] + part[1][c]) + part[2][c]) + part[3][c];
}

constexpr size_t kInferSmem = (size_t)kLayers * 64 * kRow * 2 + 4 * 16 * kRow * 2;
constexpr size_t kTrainSmem = (size_t)2 * kLayers * 64 * kRow * 2 + 4 * 16 * kRow * 2;

}  // namespace nrc
}  // namespace gpugi

// ------------------------------------------------------------------ C ABI
// Advance the EMA step count; returns 1 / (1 - d^t) (bias correction of a
// running average started at zero).
static float ema_correction(gpugi_nrc* nn) {
    nn->emaSteps++;
    return nn->emaDecay > 0.0f ? 1.0f / (1.0f - std::pow(nn->emaDecay, (float)nn->emaSteps)) : 1.0f;
}

static gpugi_status nrc_publish(gpugi_ctx* ctx, gpugi_nrc* nn) {
    nn->emaSteps = 0;
    k_nrc_publish<<<(kParams + 255) / 256, 256, 0, ctx->stream>>>(nn->master, nn->wFwd, nn->wBwd, nn->ema, nn->wInf,
                                                                  nn->wInfT);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}

gpugi_status gpugi::nrc_infer_counted(gpugi_ctx* ctx, const gpugi_nrc* nn, const float* queries, uint64_t n,
                                      const uint32_t* count, float* out) {
    if (n == 0) return GPUGI_OK;
    if (nn->kernels == GPUGI_NRC_KERNELS_TCGEN05) {
        static bool tcAttr = false;
        if (!tcAttr) {
            GPUGI_CUDA_TRY(ctx, cudaFuncSetAttribute(k_nrc_infer_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)tci::kSmem));
            tcAttr = true;
        }
        const uint64_t tiles = (n + 127) / 128;
        const uint64_t grid = std::min<uint64_t>((uint64_t)ctx->numSMs * 3, (tiles + 1) / 2);
        k_nrc_infer_tc<<<(unsigned)grid, 256, tci::kSmem, ctx->stream>>>(queries, n, count, nn->wInfT, nn->boxMin,
                                                                         nn->boxInv, out, ctx->errWord, nn->waitNs,
                                                                         nn->stall);
        GPUGI_CUDA_TRY(ctx, cudaGetLastError());
        return GPUGI_OK;
    }
    static bool attr = false;
    if (!attr) {
        GPUGI_CUDA_TRY(ctx, cudaFuncSetAttribute(k_nrc_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem));
        attr = true;
    }
    const uint64_t tiles = (n + 15) / 16;
    uint64_t blocks = (tiles + 3) / 4;
    const uint64_t maxBlocks = (uint64_t)ctx->numSMs * 4;
    if (blocks > maxBlocks) blocks = maxBlocks;
    k_nrc_infer<<<(unsigned)blocks, 128, kInferSmem, ctx->stream>>>(queries, n, count, nn->wInf, nn->boxMin,
                                                                    nn->boxInv, out);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}

extern "C" {
static gpugi_status nrc_grad(gpugi_ctx* ctx, gpugi_nrc* nn, const float* samples, uint64_t n, float* predOut,
                             const uint32_t* count);
}

// One Adam step on min(*count, cap) device samples, without a host round trip.
gpugi_status gpugi::nrc_train_counted(gpugi_ctx* ctx, gpugi_nrc* nn, const float* samples, uint64_t cap,
                                      const uint32_t* count) {
    if (cap == 0) return GPUGI_OK;
    gpugi_status st = nrc_grad(ctx, nn, samples, cap, nullptr, count);
    if (st) return st;
    nn->step++;
    const float c1 = 1.0f - std::pow(nn->beta1, (float)nn->step), c2 = 1.0f - std::pow(nn->beta2, (float)nn->step);
    const float emaCorr = ema_correction(nn);
    k_nrc_adam<<<(kParams + 255) / 256, 256, 0, ctx->stream>>>(nn->master, nn->m, nn->v, nn->grad, 0.0f, count, cap,
                                                                nn->lossScale, nn->lr, nn->beta1, nn->beta2, nn->eps,
                                                                c1, c2, nn->wFwd, nn->wBwd, nn->ema, nn->emaDecay,
                                                                emaCorr, nn->wInf, nn->wInfT);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}

extern "C" {

gpugi_status gpugi_nrc_create(gpugi_ctx* ctx, const float boxMin[3], const float boxMax[3], uint64_t seed,
                              float learningRate, gpugi_nrc** out) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!boxMin || !boxMax || !out) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    gpugi_nrc* nn = new gpugi_nrc();
    attach_child(ctx, &nn->ctx);
    nn->lr = learningRate > 0.0f ? learningRate : 1e-2f;
    nn->boxMin = make_float3(boxMin[0], boxMin[1], boxMin[2]);
    float ext[3];
    for (int d = 0; d < 3; ++d) ext[d] = boxMax[d] - boxMin[d] > 1e-12f ? boxMax[d] - boxMin[d] : 1.0f;
    nn->boxInv = make_float3(1.0f / ext[0], 1.0f / ext[1], 1.0f / ext[2]);
    const size_t P = kParams;
    bool ok = cudaMalloc(&nn->master, P * 4) == cudaSuccess && cudaMalloc(&nn->m, P * 4) == cudaSuccess &&
              cudaMalloc(&nn->v, P * 4) == cudaSuccess && cudaMalloc(&nn->grad, P * 4) == cudaSuccess &&
              cudaMalloc(&nn->wFwd, P * 2) == cudaSuccess && cudaMalloc(&nn->wBwd, P * 2) == cudaSuccess &&
              cudaMalloc(&nn->ema, P * 4) == cudaSuccess && cudaMalloc(&nn->wInf, P * 2) == cudaSuccess &&
              cudaMalloc(&nn->wInfT, P * 2) == cudaSuccess &&
              cudaMalloc(&nn->lossSum, 4) == cudaSuccess;
    if (!ok) {
        gpugi_nrc_destroy(nn);
        return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "NRC allocation failed");
    }
    // Xavier-uniform initialisation from a seeded xorshift64*.
    std::vector<float> w(P);
    uint64_t s = seed ? seed : 0x2545F4914F6CDD1DULL;
    for (int l = 0; l < kLayers; ++l) {
        const float lim = std::sqrt(6.0f / (float)(kIn + out_of(l)));
        for (int i = 0; i < kIn * out_of(l); ++i) {
            s ^= s >> 12;
            s ^= s << 25;
            s ^= s >> 27;
            const float u = (float)((s * 2685821657736338717ULL) >> 40) / 16777216.0f;
            w[layer_offset(l) + i] = (2.0f * u - 1.0f) * lim;
        }
    }
    cudaError_t e = cudaMemcpyAsync(nn->master, w.data(), P * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(nn->m, 0, P * 4, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(nn->v, 0, P * 4, ctx->stream);
    gpugi_status st = e == cudaSuccess ? nrc_publish(ctx, nn) : cuda_fail(ctx, e, "NRC initialisation");
    if (!st && (e = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) st = cuda_fail(ctx, e, "NRC initialisation");
    if (st) {
        gpugi_nrc_destroy(nn);
        return st;
    }
    *out = nn;
    return GPUGI_OK;
}

void gpugi_nrc_destroy(gpugi_nrc* nn) {
    if (!nn) return;
    if (nn->ctx) cudaStreamSynchronize(nn->ctx->stream);
    detach_child(&nn->ctx);
    for (void* p : {(void*)nn->master, (void*)nn->m, (void*)nn->v, (void*)nn->grad, (void*)nn->wFwd, (void*)nn->wBwd,
                    (void*)nn->ema, (void*)nn->wInf, (void*)nn->wInfT,
                    (void*)nn->acts, (void*)nn->dys, (void*)nn->lossSum, (void*)nn->partials})
        if (p) cudaFree(p);
    delete nn;
}

gpugi_status gpugi_nrc_get_weights(gpugi_ctx* ctx, const gpugi_nrc* nn, float* w) {
    if (!ctx || !nn || !w) return GPUGI_ERROR_INVALID_ARGUMENT;
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(w, nn->master, kParams * 4, cudaMemcpyDeviceToHost, ctx->stream));
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return GPUGI_OK;
}

gpugi_status gpugi_nrc_set_weights(gpugi_ctx* ctx, gpugi_nrc* nn, const float* w) {
    if (!ctx || !nn || !w) return GPUGI_ERROR_INVALID_ARGUMENT;
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(nn->master, w, kParams * 4, cudaMemcpyHostToDevice, ctx->stream));
    gpugi_status st = nrc_publish(ctx, nn);
    if (st) return st;
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    return GPUGI_OK;
}

gpugi_status gpugi_nrc_set_kernels(gpugi_ctx* ctx, gpugi_nrc* nn, uint32_t kernels) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!nn || kernels > GPUGI_NRC_KERNELS_MMA_SYNC) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "bad argument");
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    nn->kernels = kernels;
    return GPUGI_OK;
}

gpugi_status gpugi_nrc_debug_stall(gpugi_ctx* ctx, gpugi_nrc* nn, uint32_t stall, uint64_t waitNs) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!nn) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "bad argument");
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    nn->stall = stall ? 1u : 0u;
    nn->waitNs = waitNs ? waitNs : 1000000000ull;
    return GPUGI_OK;
}

gpugi_status gpugi_nrc_set_ema(gpugi_ctx* ctx, gpugi_nrc* nn, float decay) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!nn || !(decay >= 0.0f && decay < 1.0f)) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "decay in [0, 1)");
    nn->emaDecay = decay;
    return nrc_publish(ctx, nn);
}

gpugi_status gpugi_nrc_infer_device(gpugi_ctx* ctx, const gpugi_nrc* nn, const float* queries, uint64_t n,
                                    float* radiance) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!nn || (n && (!queries || !radiance))) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    return nrc_infer_counted(ctx, nn, queries, n, nullptr, radiance);
}

static gpugi_status nrc_grad(gpugi_ctx* ctx, gpugi_nrc* nn, const float* samples, uint64_t n, float* predOut,
                             const uint32_t* count = nullptr) {
    if (nn->kernels == GPUGI_NRC_KERNELS_TCGEN05) {
        if (!nn->partials && cudaMalloc(&nn->partials, (size_t)ctx->numSMs * kParams * 4) != cudaSuccess) {
            nn->partials = nullptr;
            return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "NRC weight-gradient partial sums");
        }
        static bool tcAttr = false;
        if (!tcAttr) {
            GPUGI_CUDA_TRY(ctx, cudaFuncSetAttribute(k_nrc_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                     (int)tcl::kSmem));
            tcAttr = true;
        }
        GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(nn->lossSum, 0, 4, ctx->stream));
        const uint64_t tiles = (n + 127) / 128;
        const int grid = (int)std::min<uint64_t>((uint64_t)ctx->numSMs, std::max<uint64_t>(tiles, 1));
        k_nrc_train_tc<<<grid, 128, tcl::kSmem, ctx->stream>>>(samples, n, count, nn->wBwd, nn->boxMin, nn->boxInv,
                                                               nn->lossScale, nn->partials, nn->lossSum, predOut,
                                                               ctx->errWord, nn->waitNs, nn->stall);
        GPUGI_CUDA_TRY(ctx, cudaGetLastError());
        k_nrc_sum_partials<<<(kParams + 63) / 64, 256, 0, ctx->stream>>>(nn->partials, grid, nn->grad);
        GPUGI_CUDA_TRY(ctx, cudaGetLastError());
        return GPUGI_OK;
    }
    if (n > nn->cap) {
        if (nn->acts) cudaFree(nn->acts);
        if (nn->dys) cudaFree(nn->dys);
        nn->acts = nn->dys = nullptr;
        nn->cap = 0;
        const uint64_t cap = (n + 15) / 16 * 16;
        if (cudaMalloc(&nn->acts, cap * kLayers * 64 * 2) != cudaSuccess ||
            cudaMalloc(&nn->dys, cap * kLayers * 64 * 2) != cudaSuccess)
            return fail(ctx, GPUGI_ERROR_OUT_OF_MEMORY, "NRC training buffers");
        nn->cap = cap;
    }
    static bool attr = false;
    if (!attr) {
        GPUGI_CUDA_TRY(ctx, cudaFuncSetAttribute(k_nrc_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTrainSmem));
        attr = true;
    }
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(nn->grad, 0, kParams * 4, ctx->stream));
    GPUGI_CUDA_TRY(ctx, cudaMemsetAsync(nn->lossSum, 0, 4, ctx->stream));
    const uint64_t tiles = (n + 15) / 16;
    uint64_t blocks = (tiles + 3) / 4;
    const uint64_t maxBlocks = (uint64_t)ctx->numSMs * 2;
    if (blocks > maxBlocks) blocks = maxBlocks;
    k_nrc_fwd_bwd<<<(unsigned)blocks, 128, kTrainSmem, ctx->stream>>>(samples, n, count, nn->wFwd, nn->wBwd, nn->boxMin,
                                                                      nn->boxInv, nn->lossScale, nn->acts, nn->dys,
                                                                      nn->cap, nn->lossSum, predOut);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    // Rows of the last partial tile beyond n were stored as zero inputs /
    // zero gradients, so the GEMM may run over whole tiles.
    uint64_t gb = (n + 511) / 512;
    if (gb > (uint64_t)ctx->numSMs) gb = ctx->numSMs;
    k_nrc_weight_grad<<<dim3((unsigned)gb, kLayers), 128, 0, ctx->stream>>>(nn->acts, nn->dys, (n + 15) / 16 * 16,
                                                                           count, nn->cap, nn->grad);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}

gpugi_status gpugi_nrc_train_device(gpugi_ctx* ctx, gpugi_nrc* nn, const float* samples, uint64_t n, float* loss) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!nn || (n && !samples)) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    if (n == 0) return GPUGI_OK;
    gpugi_status st = nrc_grad(ctx, nn, samples, n, nullptr);
    if (st) return st;
    nn->step++;
    const float c1 = 1.0f - std::pow(nn->beta1, (float)nn->step), c2 = 1.0f - std::pow(nn->beta2, (float)nn->step);
    const float gradScale = 1.0f / (3.0f * (float)n * nn->lossScale);
    const float emaCorr = ema_correction(nn);
    k_nrc_adam<<<(kParams + 255) / 256, 256, 0, ctx->stream>>>(nn->master, nn->m, nn->v, nn->grad, gradScale, nullptr,
                                                                n, nn->lossScale, nn->lr, nn->beta1, nn->beta2, nn->eps,
                                                                c1, c2, nn->wFwd, nn->wBwd, nn->ema, nn->emaDecay,
                                                                emaCorr, nn->wInf, nn->wInfT);
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    if (loss) {
        GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(loss, nn->lossSum, 4, cudaMemcpyDeviceToHost, ctx->stream));
        GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    return GPUGI_OK;
}

gpugi_status gpugi_nrc_gradient_device(gpugi_ctx* ctx, gpugi_nrc* nn, const float* samples, uint64_t n,
                                       float* predictions, float* gradient, float* loss) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!nn || !samples || !gradient || n == 0) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "bad argument");
    gpugi_status st = nrc_grad(ctx, nn, samples, n, predictions);
    if (st) return st;
    GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(gradient, nn->grad, kParams * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (loss) GPUGI_CUDA_TRY(ctx, cudaMemcpyAsync(loss, nn->lossSum, 4, cudaMemcpyDeviceToHost, ctx->stream));
    GPUGI_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    const float inv = 1.0f / (3.0f * (float)n * nn->lossScale);
    for (int i = 0; i < kParams; ++i) gradient[i] *= inv;
    return GPUGI_OK;
}

gpugi_status gpugi_nrc_encode_device(gpugi_ctx* ctx, const gpugi_nrc* nn, const float* queries, uint64_t n,
                                     void* encodedHalf) {
    if (!ctx) return GPUGI_ERROR_INVALID_ARGUMENT;
    if (!nn || (n && (!queries || !encodedHalf))) return fail(ctx, GPUGI_ERROR_INVALID_ARGUMENT, "NULL argument");
    if (n == 0) return GPUGI_OK;
    k_nrc_encode<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(queries, n, nn->boxMin, nn->boxInv,
                                                                      static_cast<__half*>(encodedHalf));
    GPUGI_CUDA_TRY(ctx, cudaGetLastError());
    return GPUGI_OK;
}

}  // extern "C"
