// The learned warm start of adjustVelocities: a small MLP on tensor cores.
//
// Per contact, 18 float32 features (below) -> 64 -> 64 -> 64 -> 3 with ReLU,
// BF16 weights and activations, FP32 accumulation, mma.sync.m16n8k16.  The
// output is the contact-frame impulse the plain resolver would apply to the
// contact in total during adjustVelocities (contact.go:388-445); applying the
// predictions first leaves the plain resolver less to do, and it still runs
// to the reference's epsilons afterwards.
//
// A 16-contact tile runs all four layers in registers: the accumulator
// fragment of an m16n8 MMA pair (columns 8j..8j+15) is, element for element,
// the A fragment of the next layer's k-step j, so a layer's output feeds the
// next layer after bias, ReLU and a round to BF16, with no data movement.
#pragma once
#include <cuda_bf16.h>

#include <cstdint>

namespace cz {

constexpr int MLP_IN = 18;   // features per contact
constexpr int MLP_H = 64;    // hidden width
constexpr int MLP_OUT = 3;   // contact-frame impulse
constexpr int MLP_K1 = 32;   // input width padded to two k-steps
constexpr int MLP_N4 = 8;    // output width padded to one n-tile
// flat float32 parameter blob (host and device master copy)
constexpr int MLP_OFF_W1 = 0;                          // [64][18]
constexpr int MLP_OFF_B1 = MLP_OFF_W1 + MLP_H * MLP_IN;  // [64]
constexpr int MLP_OFF_W2 = MLP_OFF_B1 + MLP_H;         // [64][64]
constexpr int MLP_OFF_B2 = MLP_OFF_W2 + MLP_H * MLP_H;
constexpr int MLP_OFF_W3 = MLP_OFF_B2 + MLP_H;
constexpr int MLP_OFF_B3 = MLP_OFF_W3 + MLP_H * MLP_H;
constexpr int MLP_OFF_W4 = MLP_OFF_B3 + MLP_H;         // [3][64]
constexpr int MLP_OFF_B4 = MLP_OFF_W4 + MLP_OUT * MLP_H;
constexpr int MLP_NPARAM = MLP_OFF_B4 + MLP_OUT;       // trainable parameters (9539)
constexpr int MLP_OFF_MU = MLP_NPARAM;                 // [18] feature mean
constexpr int MLP_OFF_IS = MLP_OFF_MU + MLP_IN;        // [18] 1 / feature std
constexpr int MLP_OFF_OS = MLP_OFF_IS + MLP_IN;        // [3]  output scale
constexpr int MLP_BLOB = MLP_OFF_OS + MLP_OUT;         // 9578 floats

// Device copy used by the kernels: BF16 weights in the layouts the MMA
// fragments read (row = output, column = input, zero padded), their
// transposes for the backward pass, FP32 biases and normalisation.
struct MlpDev {
  const __nv_bfloat16* W1;   // [64][32]
  const __nv_bfloat16* W2;   // [64][64]
  const __nv_bfloat16* W3;   // [64][64]
  const __nv_bfloat16* W4;   // [8][64]
  const __nv_bfloat16* W2t;  // [64][64] transposes (backward)
  const __nv_bfloat16* W3t;  // [64][64]
  const __nv_bfloat16* W4t;  // [64][16]  (columns 3..15 zero)
  const float* b1;           // [64]
  const float* b2;
  const float* b3;
  const float* b4;           // [8]
  const float* mu;           // [18]
  const float* inv_sigma;    // [18]
  const float* out_scale;    // [3]
  const float* zero;         // [64] zeros (bias of the backward GEMMs)
};

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ unsigned pack_bf16(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<unsigned*>(&v);
}

// One dense layer on a 16-row tile: c[j] (n-tile j) = bias + A . W^T, where
// W is row-major [NT*8][KS*16] BF16 (row = output).  B fragment of (k-step
// s, n-tile j): W[8j + g][16s + 2t .. +1] and W[8j + g][16s + 8 + 2t .. +1].
template <int KS, int NT>
__device__ __forceinline__ void mlp_layer(const unsigned (&a)[KS][4], const __nv_bfloat16* __restrict__ W,
                                          const float* __restrict__ bias, float (&c)[NT][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  constexpr int K = KS * 16;
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    const float bl = bias[8 * j + 2 * t], bh = bias[8 * j + 2 * t + 1];
    c[j][0] = bl; c[j][1] = bh; c[j][2] = bl; c[j][3] = bh;
    const unsigned* row = reinterpret_cast<const unsigned*>(W + (8 * j + g) * K);
#pragma unroll
    for (int s = 0; s < KS; ++s) {
      const unsigned b0 = row[8 * s + t];  // global or shared weights
      const unsigned b1 = row[8 * s + 4 + t];
      mma_bf16_16816(c[j], a[s], b0, b1);
    }
  }
}

// ReLU and round to BF16: the accumulators of n-tiles 2s, 2s+1 are the A
// fragment of k-step s of the next layer.
template <int NT>
__device__ __forceinline__ void relu_to_a(const float (&c)[NT][4], unsigned (&a)[NT / 2][4]) {
#pragma unroll
  for (int s = 0; s < NT / 2; ++s) {
    a[s][0] = pack_bf16(fmaxf(c[2 * s][0], 0.f), fmaxf(c[2 * s][1], 0.f));
    a[s][1] = pack_bf16(fmaxf(c[2 * s][2], 0.f), fmaxf(c[2 * s][3], 0.f));
    a[s][2] = pack_bf16(fmaxf(c[2 * s + 1][0], 0.f), fmaxf(c[2 * s + 1][1], 0.f));
    a[s][3] = pack_bf16(fmaxf(c[2 * s + 1][2], 0.f), fmaxf(c[2 * s + 1][3], 0.f));
  }
}

// A fragments of a 16-row tile held row-major in shared memory as BF16 [16][ld].
template <int KS>
__device__ __forceinline__ void load_a(const __nv_bfloat16* X, int ld, unsigned (&a)[KS][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int s = 0; s < KS; ++s) {
    a[s][0] = *reinterpret_cast<const unsigned*>(X + g * ld + 16 * s + 2 * t);
    a[s][1] = *reinterpret_cast<const unsigned*>(X + (g + 8) * ld + 16 * s + 2 * t);
    a[s][2] = *reinterpret_cast<const unsigned*>(X + g * ld + 16 * s + 8 + 2 * t);
    a[s][3] = *reinterpret_cast<const unsigned*>(X + (g + 8) * ld + 16 * s + 8 + 2 * t);
  }
}

// A fragments of a 16-row tile whose rows live in lanes 0..15 (row[j] = the
// lane's own BF16 pair j, columns 2j and 2j + 1), moved by warp shuffles:
// lane (g, t) takes pairs 8s + t and 8s + 4 + t of rows g and g + 8.  Every
// lane of the warp calls it.
__device__ __forceinline__ void rows_to_a(const unsigned (&row)[16], unsigned (&a)[2][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
#pragma unroll
    for (int s = 0; s < 2; ++s) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const unsigned lo = __shfl_sync(0xffffffffu, row[8 * s + 4 * h + j], g);
        const unsigned hi = __shfl_sync(0xffffffffu, row[8 * s + 4 * h + j], g + 8);
        if (t == j) {
          a[s][2 * h] = lo;
          a[s][2 * h + 1] = hi;
        }
      }
    }
  }
}

// The three outputs of row `lane & 15` from the accumulators of n-tile 0
// (row g: o[0], o[1] at columns 2t, 2t + 1; row g + 8: o[2], o[3]).  Every
// lane of the warp calls it.
__device__ __forceinline__ void out_to_rows(const float (&o)[4], float (&y)[3]) {
  const int r = threadIdx.x & 15;
  const int src = 4 * (r & 7);
  const float c00 = __shfl_sync(0xffffffffu, o[0], src), c01 = __shfl_sync(0xffffffffu, o[1], src);
  const float c20 = __shfl_sync(0xffffffffu, o[2], src), c21 = __shfl_sync(0xffffffffu, o[3], src);
  const float d0 = __shfl_sync(0xffffffffu, o[0], src + 1), d2 = __shfl_sync(0xffffffffu, o[2], src + 1);
  y[0] = r < 8 ? c00 : c20;
  y[1] = r < 8 ? c01 : c21;
  y[2] = r < 8 ? d0 : d2;
}

// Forward pass of a 16-row tile: input A fragments (normalised features as
// BF16, K padded to 32) -> output accumulators out[4] of n-tile 0 (columns
// 2t, 2t+1 of rows g and g+8; columns 0..2 are the normalised impulse).
__device__ __forceinline__ void mlp_forward_tile(const MlpDev& m, const unsigned (&x)[2][4], float (&out)[4]) {
  float h[8][4];
  unsigned a[4][4];
  mlp_layer<2, 8>(x, m.W1, m.b1, h);
  relu_to_a<8>(h, a);
  mlp_layer<4, 8>(a, m.W2, m.b2, h);
  relu_to_a<8>(h, a);
  mlp_layer<4, 8>(a, m.W3, m.b3, h);
  relu_to_a<8>(h, a);
  float o[1][4];
  mlp_layer<4, 1>(a, m.W4, m.b4, o);
  out[0] = o[0][0]; out[1] = o[0][1]; out[2] = o[0][2]; out[3] = o[0][3];
}

}  // namespace cz
