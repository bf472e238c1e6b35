// Training and inference of the warm-start MLP (cz_mlp_* in cubez_gpu.h).
//
// Parameters live as a float32 master blob (layout in cz_mlp.cuh); the kernels
// read a packed copy: BF16 weights zero-padded to the MMA tile shapes, their
// transposes for the backward pass, float32 biases and normalisation.  Every
// GEMM -- forward, backward and the weight gradients -- is mma.sync
// m16n8k16 BF16 x BF16 -> FP32 on a 16-row tile of contacts per warp.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/cubez_gpu.h"
#include "cz_forms.h"
#include "cz_mlp.cuh"

namespace cz {

// byte offsets of the packed device copy
constexpr size_t PK_W1 = 0;                                  // [64][32] bf16
constexpr size_t PK_W2 = PK_W1 + 64 * 32 * 2;                // [64][64]
constexpr size_t PK_W3 = PK_W2 + 64 * 64 * 2;
constexpr size_t PK_W4 = PK_W3 + 64 * 64 * 2;                // [8][64]
constexpr size_t PK_W2T = PK_W4 + 8 * 64 * 2;                // [64][64]
constexpr size_t PK_W3T = PK_W2T + 64 * 64 * 2;
constexpr size_t PK_W4T = PK_W3T + 64 * 64 * 2;              // [64][16]
constexpr size_t PK_B1 = PK_W4T + 64 * 16 * 2;               // f32 [64]
constexpr size_t PK_B2 = PK_B1 + 64 * 4;
constexpr size_t PK_B3 = PK_B2 + 64 * 4;
constexpr size_t PK_B4 = PK_B3 + 64 * 4;                     // [8]
constexpr size_t PK_MU = PK_B4 + 8 * 4;                      // [18]
constexpr size_t PK_IS = PK_MU + 32 * 4;                     // [18]
constexpr size_t PK_OS = PK_IS + 32 * 4;                     // [3]
constexpr size_t PK_ZERO = PK_OS + 8 * 4;                    // [64] zero bias
constexpr size_t PK_BYTES = PK_ZERO + 64 * 4;

size_t mlp_packed_bytes() { return PK_BYTES; }

MlpDev mlp_view(unsigned char* p) {
  MlpDev m;
  m.W1 = reinterpret_cast<const __nv_bfloat16*>(p + PK_W1);
  m.W2 = reinterpret_cast<const __nv_bfloat16*>(p + PK_W2);
  m.W3 = reinterpret_cast<const __nv_bfloat16*>(p + PK_W3);
  m.W4 = reinterpret_cast<const __nv_bfloat16*>(p + PK_W4);
  m.W2t = reinterpret_cast<const __nv_bfloat16*>(p + PK_W2T);
  m.W3t = reinterpret_cast<const __nv_bfloat16*>(p + PK_W3T);
  m.W4t = reinterpret_cast<const __nv_bfloat16*>(p + PK_W4T);
  m.b1 = reinterpret_cast<const float*>(p + PK_B1);
  m.b2 = reinterpret_cast<const float*>(p + PK_B2);
  m.b3 = reinterpret_cast<const float*>(p + PK_B3);
  m.b4 = reinterpret_cast<const float*>(p + PK_B4);
  m.mu = reinterpret_cast<const float*>(p + PK_MU);
  m.inv_sigma = reinterpret_cast<const float*>(p + PK_IS);
  m.out_scale = reinterpret_cast<const float*>(p + PK_OS);
  m.zero = reinterpret_cast<const float*>(p + PK_ZERO);
  return m;
}

// master blob -> packed copy
__global__ void k_mlp_pack(const float* __restrict__ blob, unsigned char* __restrict__ p) {
  __nv_bfloat16* W1 = reinterpret_cast<__nv_bfloat16*>(p + PK_W1);
  __nv_bfloat16* W2 = reinterpret_cast<__nv_bfloat16*>(p + PK_W2);
  __nv_bfloat16* W3 = reinterpret_cast<__nv_bfloat16*>(p + PK_W3);
  __nv_bfloat16* W4 = reinterpret_cast<__nv_bfloat16*>(p + PK_W4);
  __nv_bfloat16* W2t = reinterpret_cast<__nv_bfloat16*>(p + PK_W2T);
  __nv_bfloat16* W3t = reinterpret_cast<__nv_bfloat16*>(p + PK_W3T);
  __nv_bfloat16* W4t = reinterpret_cast<__nv_bfloat16*>(p + PK_W4T);
  float* b = reinterpret_cast<float*>(p + PK_B1);
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nt = gridDim.x * blockDim.x;
  for (int i = tid; i < 64 * 32; i += nt) {
    const int o = i / 32, c = i % 32;
    W1[i] = __float2bfloat16_rn(c < MLP_IN ? blob[MLP_OFF_W1 + o * MLP_IN + c] : 0.f);
  }
  for (int i = tid; i < 64 * 64; i += nt) {
    const int o = i / 64, c = i % 64;
    W2[i] = __float2bfloat16_rn(blob[MLP_OFF_W2 + i]);
    W3[i] = __float2bfloat16_rn(blob[MLP_OFF_W3 + i]);
    W2t[c * 64 + o] = __float2bfloat16_rn(blob[MLP_OFF_W2 + i]);
    W3t[c * 64 + o] = __float2bfloat16_rn(blob[MLP_OFF_W3 + i]);
  }
  for (int i = tid; i < 8 * 64; i += nt) {
    const int o = i / 64, c = i % 64;
    W4[i] = __float2bfloat16_rn(o < MLP_OUT ? blob[MLP_OFF_W4 + o * 64 + c] : 0.f);
  }
  for (int i = tid; i < 64 * 16; i += nt) {
    const int c = i / 16, o = i % 16;  // W4t[in][out]
    W4t[i] = __float2bfloat16_rn(o < MLP_OUT ? blob[MLP_OFF_W4 + o * 64 + c] : 0.f);
  }
  for (int i = tid; i < 64; i += nt) {
    b[i] = blob[MLP_OFF_B1 + i];
    b[64 + i] = blob[MLP_OFF_B2 + i];
    b[128 + i] = blob[MLP_OFF_B3 + i];
    reinterpret_cast<float*>(p + PK_ZERO)[i] = 0.f;
  }
  for (int i = tid; i < 8; i += nt) reinterpret_cast<float*>(p + PK_B4)[i] = i < MLP_OUT ? blob[MLP_OFF_B4 + i] : 0.f;
  for (int i = tid; i < MLP_IN; i += nt) {
    reinterpret_cast<float*>(p + PK_MU)[i] = blob[MLP_OFF_MU + i];
    reinterpret_cast<float*>(p + PK_IS)[i] = blob[MLP_OFF_IS + i];
  }
  for (int i = tid; i < MLP_OUT; i += nt) reinterpret_cast<float*>(p + PK_OS)[i] = blob[MLP_OFF_OS + i];
}

cudaError_t mlp_pack(const float* dev_blob, unsigned char* dev_packed, cudaStream_t s) {
  k_mlp_pack<<<8, 256, 0, s>>>(dev_blob, dev_packed);
  return cudaGetLastError();
}

namespace {

constexpr int kTrainWarps = 4;
// per-warp staging in shared memory: input, three activations, one gradient tile
constexpr int kStageX = 16 * MLP_K1;   // bf16
constexpr int kStageH = 16 * MLP_H;    // bf16
constexpr int kWarpStage = kStageX + 4 * kStageH;  // bf16 elements

__device__ __forceinline__ unsigned short bf16_bits(float f) {
  __nv_bfloat16 b = __float2bfloat16_rn(f);
  return *reinterpret_cast<unsigned short*>(&b);
}
__device__ __forceinline__ float bf16_val(unsigned short u) {
  return __uint_as_float(((unsigned)u) << 16);
}

// write a 16x(8*NT) accumulator tile to shared memory as BF16 [16][ld]
template <int NT>
__device__ __forceinline__ void store_tile(const float (&c)[NT][4], unsigned short* S, int ld) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    S[g * ld + 8 * j + 2 * t] = bf16_bits(c[j][0]);
    S[g * ld + 8 * j + 2 * t + 1] = bf16_bits(c[j][1]);
    S[(g + 8) * ld + 8 * j + 2 * t] = bf16_bits(c[j][2]);
    S[(g + 8) * ld + 8 * j + 2 * t + 1] = bf16_bits(c[j][3]);
  }
}

// dW[out][in] += sum over the 16 rows of dZ[row][out] * H[row][in]: one MMA per
// (16 outputs x 8 inputs) tile with the rows as the reduction; dZ and H are
// BF16 [16][ld] in shared memory; the result is added into g (shared, row
// length in_len, only out < out_len and in < in_len kept).
__device__ void weight_grad(const unsigned short* dZ, int ldz, int out_pad, const unsigned short* H, int ldh,
                            int in_pad, float* g, int out_len, int in_len) {
  const int lane = threadIdx.x & 31, gr = lane >> 2, t = lane & 3;
  for (int mi = 0; mi < out_pad / 16; ++mi) {
    unsigned a[4];
    // A[m = out][k = row] = dZ[row][out]
    auto A = [&](int m, int k) { return (unsigned)dZ[k * ldz + 16 * mi + m]; };
    a[0] = A(gr, 2 * t) | (A(gr, 2 * t + 1) << 16);
    a[1] = A(gr + 8, 2 * t) | (A(gr + 8, 2 * t + 1) << 16);
    a[2] = A(gr, 2 * t + 8) | (A(gr, 2 * t + 9) << 16);
    a[3] = A(gr + 8, 2 * t + 8) | (A(gr + 8, 2 * t + 9) << 16);
    for (int nj = 0; nj < in_pad / 8; ++nj) {
      // B[k = row][n = in] = H[row][in]
      auto B = [&](int k, int n) { return (unsigned)H[k * ldh + 8 * nj + n]; };
      const unsigned b0 = B(2 * t, gr) | (B(2 * t + 1, gr) << 16);
      const unsigned b1 = B(2 * t + 8, gr) | (B(2 * t + 9, gr) << 16);
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      mma_bf16_16816(d, a, b0, b1);
      const int o0 = 16 * mi + gr, o1 = o0 + 8, i0 = 8 * nj + 2 * t;
      if (o0 < out_len && i0 < in_len) atomicAdd(&g[o0 * in_len + i0], d[0]);
      if (o0 < out_len && i0 + 1 < in_len) atomicAdd(&g[o0 * in_len + i0 + 1], d[1]);
      if (o1 < out_len && i0 < in_len) atomicAdd(&g[o1 * in_len + i0], d[2]);
      if (o1 < out_len && i0 + 1 < in_len) atomicAdd(&g[o1 * in_len + i0 + 1], d[3]);
    }
  }
}

// bias gradient: column sums of a 16-row accumulator tile
template <int NT> __device__ __forceinline__ void bias_grad(const float (&c)[NT][4], float* g, int len) {
  const int lane = threadIdx.x & 31, t = lane & 3;
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    float s0 = c[j][0] + c[j][2], s1 = c[j][1] + c[j][3];
#pragma unroll
    for (int off = 4; off < 32; off <<= 1) {
      s0 += __shfl_xor_sync(0xffffffffu, s0, off);
      s1 += __shfl_xor_sync(0xffffffffu, s1, off);
    }
    if (lane < 4) {
      if (8 * j + 2 * t < len) atomicAdd(&g[8 * j + 2 * t], s0);
      if (8 * j + 2 * t + 1 < len) atomicAdd(&g[8 * j + 2 * t + 1], s1);
    }
  }
}

template <int NT>
__device__ __forceinline__ void relu_mask(float (&c)[NT][4], const unsigned short* H, int ld) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    if (!(bf16_val(H[g * ld + 8 * j + 2 * t]) > 0.f)) c[j][0] = 0.f;
    if (!(bf16_val(H[g * ld + 8 * j + 2 * t + 1]) > 0.f)) c[j][1] = 0.f;
    if (!(bf16_val(H[(g + 8) * ld + 8 * j + 2 * t]) > 0.f)) c[j][2] = 0.f;
    if (!(bf16_val(H[(g + 8) * ld + 8 * j + 2 * t + 1]) > 0.f)) c[j][3] = 0.f;
  }
}

template <int NT> __device__ __forceinline__ void to_a(const float (&c)[NT][4], unsigned (&a)[NT / 2][4]) {
#pragma unroll
  for (int s = 0; s < NT / 2; ++s) {
    a[s][0] = pack_bf16(c[2 * s][0], c[2 * s][1]);
    a[s][1] = pack_bf16(c[2 * s][2], c[2 * s][3]);
    a[s][2] = pack_bf16(c[2 * s + 1][0], c[2 * s + 1][1]);
    a[s][3] = pack_bf16(c[2 * s + 1][2], c[2 * s + 1][3]);
  }
}

// Forward + backward over tiles of 16 rows (rows idx[r] of x, y; n rows in
// total); mean squared error of the normalised outputs.  Gradients are summed
// in shared memory per CTA, then added to grad (global); loss (sum) likewise.
__global__ void __launch_bounds__(kTrainWarps * 32)
    k_mlp_train(MlpDev m, const float* __restrict__ x, const float* __restrict__ y, const int* __restrict__ idx,
                long long n, float scale, float* __restrict__ grad, float* __restrict__ loss) {
  extern __shared__ __align__(16) unsigned char sm[];
  float* gs = reinterpret_cast<float*>(sm);  // [MLP_NPARAM] gradient accumulators
  float* ls = gs + MLP_NPARAM;               // loss accumulator
  unsigned short* stage =
      reinterpret_cast<unsigned short*>(ls + 4) + (threadIdx.x >> 5) * kWarpStage;
  unsigned short* X = stage;
  unsigned short* H1 = X + kStageX;
  unsigned short* H2 = H1 + kStageH;
  unsigned short* H3 = H2 + kStageH;
  unsigned short* DZ = H3 + kStageH;
  for (int i = threadIdx.x; i < MLP_NPARAM + 4; i += blockDim.x) gs[i] = 0.f;
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const long long tiles = (n + 15) / 16;
  const long long warp = (long long)blockIdx.x * kTrainWarps + (threadIdx.x >> 5);
  const long long nwarps = (long long)gridDim.x * kTrainWarps;
  float lsum = 0.f;
  for (long long tile = warp; tile < tiles; tile += nwarps) {
    // normalised inputs (BF16) of the tile's rows
    if (lane < 16) {
      const long long r = tile * 16 + lane;
      const long long row = r < n ? idx[r] : -1;
      for (int c = 0; c < MLP_K1; ++c) {
        float v = 0.f;
        if (row >= 0 && c < MLP_IN) v = (x[row * MLP_IN + c] - m.mu[c]) * m.inv_sigma[c];
        X[lane * MLP_K1 + c] = bf16_bits(v);
      }
    }
    __syncwarp();
    unsigned ax[2][4];
    load_a<2>(reinterpret_cast<const __nv_bfloat16*>(X), MLP_K1, ax);
    float h[8][4];
    unsigned a[4][4];
    mlp_layer<2, 8>(ax, m.W1, m.b1, h);
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) h[j][q] = fmaxf(h[j][q], 0.f);
    store_tile<8>(h, H1, MLP_H);
    to_a<8>(h, a);
    mlp_layer<4, 8>(a, m.W2, m.b2, h);
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) h[j][q] = fmaxf(h[j][q], 0.f);
    store_tile<8>(h, H2, MLP_H);
    to_a<8>(h, a);
    mlp_layer<4, 8>(a, m.W3, m.b3, h);
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int q = 0; q < 4; ++q) h[j][q] = fmaxf(h[j][q], 0.f);
    store_tile<8>(h, H3, MLP_H);
    to_a<8>(h, a);
    float o[1][4];
    mlp_layer<4, 1>(a, m.W4, m.b4, o);
    // loss and dL/do (rows beyond n and columns >= 3 contribute nothing)
    const long long r0 = tile * 16 + g, r1 = r0 + 8;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long r = q < 2 ? r0 : r1;
      const int col = 2 * t + (q & 1);
      float d = 0.f;
      if (r < n && col < MLP_OUT) {
        const float target = y[idx[r] * MLP_OUT + col] / m.out_scale[col];
        d = o[0][q] - target;
        lsum += d * d;
      }
      o[0][q] = 2.f * d * scale;
    }
    __syncwarp();
    // layer 4: dW4 = dO^T H3, db4 = sum dO, dH3 = dO W4
    store_tile<1>(o, DZ, 16);
    for (int i = lane; i < 16 * 8; i += 32) DZ[(i / 8) * 16 + 8 + (i % 8)] = 0;  // columns 8..15
    __syncwarp();
    bias_grad<1>(o, gs + MLP_OFF_B4, MLP_OUT);
    weight_grad(DZ, 16, 16, H3, MLP_H, 64, gs + MLP_OFF_W4, MLP_OUT, MLP_H);
    unsigned ad[1][4];
    ad[0][0] = pack_bf16(o[0][0], o[0][1]);
    ad[0][1] = pack_bf16(o[0][2], o[0][3]);
    ad[0][2] = 0u;
    ad[0][3] = 0u;
    mlp_layer<1, 8>(ad, m.W4t, m.zero, h);
    relu_mask<8>(h, H3, MLP_H);
    // layer 3
    __syncwarp();
    store_tile<8>(h, DZ, MLP_H);
    __syncwarp();
    bias_grad<8>(h, gs + MLP_OFF_B3, MLP_H);
    weight_grad(DZ, MLP_H, 64, H2, MLP_H, 64, gs + MLP_OFF_W3, MLP_H, MLP_H);
    to_a<8>(h, a);
    mlp_layer<4, 8>(a, m.W3t, m.zero, h);
    relu_mask<8>(h, H2, MLP_H);
    // layer 2
    __syncwarp();
    store_tile<8>(h, DZ, MLP_H);
    __syncwarp();
    bias_grad<8>(h, gs + MLP_OFF_B2, MLP_H);
    weight_grad(DZ, MLP_H, 64, H1, MLP_H, 64, gs + MLP_OFF_W2, MLP_H, MLP_H);
    to_a<8>(h, a);
    mlp_layer<4, 8>(a, m.W2t, m.zero, h);
    relu_mask<8>(h, H1, MLP_H);
    // layer 1
    __syncwarp();
    store_tile<8>(h, DZ, MLP_H);
    __syncwarp();
    bias_grad<8>(h, gs + MLP_OFF_B1, MLP_H);
    weight_grad(DZ, MLP_H, 64, X, MLP_K1, 32, gs + MLP_OFF_W1, MLP_H, MLP_IN);
    __syncwarp();
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, off);
  if (lane == 0) atomicAdd(ls, lsum);
  __syncthreads();
  for (int i = threadIdx.x; i < MLP_NPARAM; i += blockDim.x) atomicAdd(&grad[i], gs[i]);
  if (threadIdx.x == 0) atomicAdd(loss, ls[0]);
}

// inference of n rows: denormalised outputs
__global__ void __launch_bounds__(128) k_mlp_predict(MlpDev m, const float* __restrict__ x, long long n,
                                                     float* __restrict__ out) {
  __shared__ __align__(16) unsigned short X[4][16 * MLP_K1];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, g = lane >> 2, t = lane & 3;
  const long long tiles = (n + 15) / 16;
  for (long long tile = (long long)blockIdx.x * 4 + w; tile < tiles; tile += (long long)gridDim.x * 4) {
    if (lane < 16) {
      const long long r = tile * 16 + lane;
      for (int c = 0; c < MLP_K1; ++c) {
        float v = 0.f;
        if (r < n && c < MLP_IN) v = (x[r * MLP_IN + c] - m.mu[c]) * m.inv_sigma[c];
        X[w][lane * MLP_K1 + c] = bf16_bits(v);
      }
    }
    __syncwarp();
    unsigned a[2][4];
    load_a<2>(reinterpret_cast<const __nv_bfloat16*>(X[w]), MLP_K1, a);
    float o[4];
    mlp_forward_tile(m, a, o);
    const long long r0 = tile * 16 + g, r1 = r0 + 8;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const long long r = q < 2 ? r0 : r1;
      const int col = 2 * t + (q & 1);
      if (r < n && col < MLP_OUT) out[r * MLP_OUT + col] = o[q] * m.out_scale[col];
    }
    __syncwarp();
  }
}

// Adam on the trainable part of the master blob, then zero the gradient
__global__ void k_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m1, float* __restrict__ m2,
                       float lr, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= MLP_NPARAM) return;
  const float gi = g[i];
  const float a = 0.9f * m1[i] + 0.1f * gi;
  const float b = 0.999f * m2[i] + 0.001f * gi * gi;
  m1[i] = a;
  m2[i] = b;
  p[i] -= lr * (a / c1) / (sqrtf(b / c2) + 1e-8f);
  g[i] = 0.f;
}

constexpr size_t kTrainSmem = (MLP_NPARAM + 4) * 4 + kTrainWarps * kWarpStage * 2;

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace
}  // namespace cz

struct cz_mlp {
  int device = 0;
  cudaStream_t stream = nullptr;
  float* master = nullptr;  // [MLP_BLOB]
  float* grad = nullptr;    // [MLP_NPARAM] (+ loss)
  float* m1 = nullptr;
  float* m2 = nullptr;
  unsigned char* packed = nullptr;
  float* x = nullptr;
  float* y = nullptr;
  int* idx = nullptr;
  long long n = 0, cap = 0;
  long long step = 0;
  int sms = 1;
};

namespace {
#define MLP_CUDA(call)                                                   \
  do {                                                                   \
    cudaError_t e_ = (call);                                             \
    if (e_ != cudaSuccess) return cz::set_error(CZ_ERR_CUDA, #call, e_); \
  } while (0)

int ensure_data(cz_mlp* m, long long n) {
  if (n <= m->cap) return CZ_OK;
  cudaFree(m->x);
  cudaFree(m->y);
  cudaFree(m->idx);
  m->x = nullptr;
  m->y = nullptr;
  m->idx = nullptr;
  m->cap = 0;
  MLP_CUDA(cudaMalloc(&m->x, sizeof(float) * cz::MLP_IN * n));
  MLP_CUDA(cudaMalloc(&m->y, sizeof(float) * cz::MLP_OUT * n));
  MLP_CUDA(cudaMalloc(&m->idx, sizeof(int) * n));
  m->cap = n;
  return CZ_OK;
}

int repack(cz_mlp* m) {
  MLP_CUDA(cz::mlp_pack(m->master, m->packed, m->stream));
  return CZ_OK;
}
}  // namespace

extern "C" {

int cz_mlp_create(int32_t device, uint64_t seed, cz_mlp** out) {
  if (!out) return cz::set_error(CZ_ERR_BAD_ARG, "cz_mlp_create: null output", cudaSuccess);
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0)
    return cz::set_error(CZ_ERR_NO_DEVICE, "no CUDA device", cudaSuccess);
  cz_mlp* m = new cz_mlp();
  m->device = device;
  auto bail = [&](int st) {
    cz_mlp_destroy(m);
    return st;
  };
  if (cudaSetDevice(device) != cudaSuccess) return bail(CZ_ERR_BAD_ARG);
  cudaDeviceGetAttribute(&m->sms, cudaDevAttrMultiProcessorCount, device);
  if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaMalloc(&m->master, sizeof(float) * cz::MLP_BLOB) != cudaSuccess ||
      cudaMalloc(&m->grad, sizeof(float) * (cz::MLP_NPARAM + 1)) != cudaSuccess ||
      cudaMalloc(&m->m1, sizeof(float) * cz::MLP_NPARAM) != cudaSuccess ||
      cudaMalloc(&m->m2, sizeof(float) * cz::MLP_NPARAM) != cudaSuccess ||
      cudaMalloc(&m->packed, cz::mlp_packed_bytes()) != cudaSuccess)
    return bail(cz::set_error(CZ_ERR_CUDA, "cz_mlp_create: allocation", cudaGetLastError()));
  // He-uniform initialisation from a seeded splitmix64 stream, zero biases,
  // identity normalisation
  std::vector<float> blob(cz::MLP_BLOB, 0.f);
  uint64_t s = seed;
  auto fill = [&](int off, int rows, int cols) {
    const float bound = std::sqrt(6.f / (float)cols);
    for (int i = 0; i < rows * cols; ++i) {
      const double u = (double)(cz::splitmix(s) >> 11) * (1.0 / 9007199254740992.0);
      blob[off + i] = (float)((2.0 * u - 1.0) * bound);
    }
  };
  fill(cz::MLP_OFF_W1, cz::MLP_H, cz::MLP_IN);
  fill(cz::MLP_OFF_W2, cz::MLP_H, cz::MLP_H);
  fill(cz::MLP_OFF_W3, cz::MLP_H, cz::MLP_H);
  fill(cz::MLP_OFF_W4, cz::MLP_OUT, cz::MLP_H);
  for (int i = 0; i < cz::MLP_IN; ++i) blob[cz::MLP_OFF_IS + i] = 1.f;
  for (int i = 0; i < cz::MLP_OUT; ++i) blob[cz::MLP_OFF_OS + i] = 1.f;
  if (cudaMemcpy(m->master, blob.data(), sizeof(float) * cz::MLP_BLOB, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemset(m->grad, 0, sizeof(float) * (cz::MLP_NPARAM + 1)) != cudaSuccess ||
      cudaMemset(m->m1, 0, sizeof(float) * cz::MLP_NPARAM) != cudaSuccess ||
      cudaMemset(m->m2, 0, sizeof(float) * cz::MLP_NPARAM) != cudaSuccess)
    return bail(cz::set_error(CZ_ERR_CUDA, "cz_mlp_create: initialisation", cudaGetLastError()));
  if (repack(m) != CZ_OK || cudaStreamSynchronize(m->stream) != cudaSuccess) return bail(CZ_ERR_CUDA);
  if (cudaFuncSetAttribute(cz::k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cz::kTrainSmem) !=
      cudaSuccess)
    return bail(cz::set_error(CZ_ERR_CUDA, "cz_mlp_create: training kernel attributes", cudaGetLastError()));
  *out = m;
  return CZ_OK;
}

int cz_mlp_destroy(cz_mlp* m) {
  if (!m) return CZ_ERR_BAD_ARG;
  cudaSetDevice(m->device);
  void* p[] = {m->master, m->grad, m->m1, m->m2, m->packed, m->x, m->y, m->idx};
  for (void* q : p)
    if (q) cudaFree(q);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return CZ_OK;
}

int cz_mlp_get_params(cz_mlp* m, float* blob) {
  if (!m || !blob) return cz::set_error(CZ_ERR_BAD_ARG, "cz_mlp_get_params: null argument", cudaSuccess);
  MLP_CUDA(cudaSetDevice(m->device));
  MLP_CUDA(cudaMemcpyAsync(blob, m->master, sizeof(float) * cz::MLP_BLOB, cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  return CZ_OK;
}

int cz_mlp_set_params(cz_mlp* m, const float* blob) {
  if (!m || !blob) return cz::set_error(CZ_ERR_BAD_ARG, "cz_mlp_set_params: null argument", cudaSuccess);
  MLP_CUDA(cudaSetDevice(m->device));
  MLP_CUDA(cudaMemcpyAsync(m->master, blob, sizeof(float) * cz::MLP_BLOB, cudaMemcpyHostToDevice, m->stream));
  int st = repack(m);
  if (st) return st;
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  return CZ_OK;
}

int cz_mlp_set_data(cz_mlp* m, const float* x, const float* y, int64_t n, int32_t set_normalization) {
  if (!m || !x || !y || n <= 0) return cz::set_error(CZ_ERR_BAD_ARG, "cz_mlp_set_data: bad argument", cudaSuccess);
  MLP_CUDA(cudaSetDevice(m->device));
  int st = ensure_data(m, n);
  if (st) return st;
  MLP_CUDA(cudaMemcpyAsync(m->x, x, sizeof(float) * cz::MLP_IN * n, cudaMemcpyHostToDevice, m->stream));
  MLP_CUDA(cudaMemcpyAsync(m->y, y, sizeof(float) * cz::MLP_OUT * n, cudaMemcpyHostToDevice, m->stream));
  m->n = n;
  if (set_normalization) {
    // feature mean / standard deviation and output scale from the data
    std::vector<float> blob(cz::MLP_BLOB);
    MLP_CUDA(cudaMemcpyAsync(blob.data(), m->master, sizeof(float) * cz::MLP_BLOB, cudaMemcpyDeviceToHost,
                             m->stream));
    MLP_CUDA(cudaStreamSynchronize(m->stream));
    for (int c = 0; c < cz::MLP_IN; ++c) {
      double s1 = 0, s2 = 0;
      for (long long r = 0; r < n; ++r) {
        const double v = x[r * cz::MLP_IN + c];
        s1 += v;
        s2 += v * v;
      }
      const double mu = s1 / n, var = std::max(s2 / n - mu * mu, 0.0);
      blob[cz::MLP_OFF_MU + c] = (float)mu;
      blob[cz::MLP_OFF_IS + c] = (float)(1.0 / std::sqrt(var + 1e-12));
      if (var < 1e-20) blob[cz::MLP_OFF_IS + c] = 0.f;  // constant feature
    }
    for (int c = 0; c < cz::MLP_OUT; ++c) {
      double s2 = 0;
      for (long long r = 0; r < n; ++r) s2 += (double)y[r * cz::MLP_OUT + c] * y[r * cz::MLP_OUT + c];
      blob[cz::MLP_OFF_OS + c] = (float)std::max(std::sqrt(s2 / n), 1e-6);
    }
    return cz_mlp_set_params(m, blob.data());
  }
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  return CZ_OK;
}

// Mean loss and gradient of the first n rows of the data set (no update).
int cz_mlp_loss_and_grad(cz_mlp* m, int64_t n, float* loss, float* grad) {
  if (!m || n <= 0 || n > m->n) return cz::set_error(CZ_ERR_BAD_ARG, "cz_mlp_loss_and_grad: bad n", cudaSuccess);
  MLP_CUDA(cudaSetDevice(m->device));
  std::vector<int> idx(n);
  for (long long i = 0; i < n; ++i) idx[i] = (int)i;
  MLP_CUDA(cudaMemcpyAsync(m->idx, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice, m->stream));
  MLP_CUDA(cudaMemsetAsync(m->grad, 0, sizeof(float) * (cz::MLP_NPARAM + 1), m->stream));
  const float scale = 1.f / (float)(cz::MLP_OUT * n);
  const int grid = (int)std::min<long long>((n + 16 * cz::kTrainWarps - 1) / (16 * cz::kTrainWarps), 4LL * m->sms);
  cz::k_mlp_train<<<grid, cz::kTrainWarps * 32, cz::kTrainSmem, m->stream>>>(
      cz::mlp_view(m->packed), m->x, m->y, m->idx, n, scale, m->grad, m->grad + cz::MLP_NPARAM);
  MLP_CUDA(cudaGetLastError());
  std::vector<float> g(cz::MLP_NPARAM + 1);
  MLP_CUDA(cudaMemcpyAsync(g.data(), m->grad, sizeof(float) * (cz::MLP_NPARAM + 1), cudaMemcpyDeviceToHost,
                           m->stream));
  MLP_CUDA(cudaMemsetAsync(m->grad, 0, sizeof(float) * (cz::MLP_NPARAM + 1), m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  if (grad) std::memcpy(grad, g.data(), sizeof(float) * cz::MLP_NPARAM);
  if (loss) *loss = g[cz::MLP_NPARAM] * scale;
  return CZ_OK;
}

// Adam over shuffled mini-batches of the data set; epoch_loss[e] = mean loss.
int cz_mlp_train(cz_mlp* m, int32_t epochs, int32_t batch, float lr, uint64_t seed, float* epoch_loss) {
  if (!m || epochs <= 0 || batch <= 0 || m->n <= 0)
    return cz::set_error(CZ_ERR_BAD_ARG, "cz_mlp_train: bad argument", cudaSuccess);
  MLP_CUDA(cudaSetDevice(m->device));
  std::vector<int> idx(m->n);
  uint64_t s = seed;
  for (int e = 0; e < epochs; ++e) {
    for (long long i = 0; i < m->n; ++i) idx[i] = (int)i;
    for (long long i = m->n - 1; i > 0; --i) std::swap(idx[i], idx[cz::splitmix(s) % (uint64_t)(i + 1)]);
    MLP_CUDA(cudaMemcpyAsync(m->idx, idx.data(), sizeof(int) * m->n, cudaMemcpyHostToDevice, m->stream));
    MLP_CUDA(cudaMemsetAsync(m->grad + cz::MLP_NPARAM, 0, sizeof(float), m->stream));
    for (long long b0 = 0; b0 < m->n; b0 += batch) {
      const long long nb = std::min<long long>(batch, m->n - b0);
      const float scale = 1.f / (float)(cz::MLP_OUT * nb);
      const int grid =
          (int)std::min<long long>((nb + 16 * cz::kTrainWarps - 1) / (16 * cz::kTrainWarps), 4LL * m->sms);
      cz::k_mlp_train<<<grid, cz::kTrainWarps * 32, cz::kTrainSmem, m->stream>>>(
          cz::mlp_view(m->packed), m->x, m->y, m->idx + b0, nb, scale, m->grad, m->grad + cz::MLP_NPARAM);
      ++m->step;
      const float c1 = 1.f - std::pow(0.9f, (float)m->step), c2 = 1.f - std::pow(0.999f, (float)m->step);
      cz::k_adam<<<(cz::MLP_NPARAM + 255) / 256, 256, 0, m->stream>>>(m->master, m->grad, m->m1, m->m2, lr, c1, c2);
      int st = repack(m);
      if (st) return st;
    }
    MLP_CUDA(cudaGetLastError());
    float lsum = 0.f;
    MLP_CUDA(cudaMemcpyAsync(&lsum, m->grad + cz::MLP_NPARAM, sizeof(float), cudaMemcpyDeviceToHost, m->stream));
    MLP_CUDA(cudaStreamSynchronize(m->stream));
    if (epoch_loss) epoch_loss[e] = lsum / (float)(cz::MLP_OUT * m->n);
  }
  return CZ_OK;
}

int cz_mlp_predict(cz_mlp* m, const float* x, int64_t n, float* out) {
  if (!m || !x || !out || n <= 0) return cz::set_error(CZ_ERR_BAD_ARG, "cz_mlp_predict: bad argument", cudaSuccess);
  MLP_CUDA(cudaSetDevice(m->device));
  float *dx = nullptr, *dy = nullptr;
  MLP_CUDA(cudaMalloc(&dx, sizeof(float) * cz::MLP_IN * n));
  if (cudaMalloc(&dy, sizeof(float) * cz::MLP_OUT * n) != cudaSuccess) {
    cudaFree(dx);
    return cz::set_error(CZ_ERR_CUDA, "cz_mlp_predict: allocation", cudaGetLastError());
  }
  cudaMemcpyAsync(dx, x, sizeof(float) * cz::MLP_IN * n, cudaMemcpyHostToDevice, m->stream);
  const int grid = (int)std::min<long long>((n + 63) / 64, 8LL * m->sms);
  cz::k_mlp_predict<<<grid, 128, 0, m->stream>>>(cz::mlp_view(m->packed), dx, n, dy);
  cudaError_t e = cudaGetLastError();
  cudaMemcpyAsync(out, dy, sizeof(float) * cz::MLP_OUT * n, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  cudaFree(dx);
  cudaFree(dy);
  if (e != cudaSuccess) return cz::set_error(CZ_ERR_CUDA, "cz_mlp_predict", e);
  return CZ_OK;
}

}  // extern "C"
