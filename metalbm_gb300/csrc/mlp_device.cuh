// Learned alpha guess fused into the entropic collide kernel.
//
// Network: x (Q features, zero-padded to 32) -> 32 -> 32 -> 1, tanh hidden
// layers; x_q = (f_neq_q / rho) * input_scale_q; guess = 2 + output_scale * y.
// Inference runs on the tensor cores as BF16 mma.sync.m16n8k16 with FP32
// accumulation, over the 128 nodes of a thread block: each warp stacks the
// feature rows of its 32 nodes (two m16 tiles) in shared memory, multiplies by
// W1^T (K = 32, N = 32: 2 k-steps x 4 n-tiles), applies bias + tanh on the
// accumulator fragments, re-uses those fragments directly as the A operand of
// the second layer (the m16n8 accumulator layout of two adjacent n-tiles is
// the m16k16 A layout), and finishes the 32-wide output dot product with
// quad shuffles.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace mlbm {

constexpr int MLP_H = 32;
constexpr int MLP_ROW = 40;  // smem row stride in bf16 (80 B: conflict-free fragment loads)

struct MlpDev {
  __nv_bfloat16 w1[MLP_H * 32];  // [hidden][in, zero padded to 32]
  __nv_bfloat16 w2[MLP_H * MLP_H];
  float b1[MLP_H];
  float b2[MLP_H];
  float w3[MLP_H];
  float in_scale[32];
  float b3;
  float out_scale;
  int n_in;
  int pad;
};

// Hardware tanh (tanh.approx.f32, one SFU instruction; absolute error
// below 2^-10, the order of the BF16 rounding of the activations). The
// library tanhf is a long FP32 instruction sequence, evaluated 64 times a
// node here; the hardware one moves the guess by ~1e-7 (output_scale x 1e-3),
// far inside the Newton acceptance window.
__device__ __forceinline__ float tanh_hw(float x) {
  float r;
  asm("tanh.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ void mma_bf16_16816(float d[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// One 32-node warp tile: rows (the warp's nodes) x features in smem -> the
// guess minus 2 (kept apart so the caller adds 2 in its own precision) for
// this thread's own node. Every lane of the warp must call it.
template <int Q>
__device__ __forceinline__ float mlp_guess_warp(const MlpDev* __restrict__ m, const float x[Q],
                                                __nv_bfloat16* rows /* 32 x MLP_ROW */,
                                                float* ysh /* 32 */) {
  const int lane = threadIdx.x & 31;
  const int g = lane >> 2, t = lane & 3;
  // stage this node's scaled features as one bf16 row
  {
    uint32_t* r = reinterpret_cast<uint32_t*>(rows + lane * MLP_ROW);
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const int q0 = 2 * k, q1 = 2 * k + 1;
      const float v0 = q0 < Q ? x[q0 < Q ? q0 : 0] * __ldg(&m->in_scale[q0]) : 0.0f;
      const float v1 = q1 < Q ? x[q1 < Q ? q1 : 0] * __ldg(&m->in_scale[q1]) : 0.0f;
      r[k] = pack_bf16(v0, v1);
    }
  }
  __syncwarp();
  float acc[2][4][4];  // [m-tile][n-tile][frag]
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const float b0 = __ldg(&m->b1[nt * 8 + 2 * t]), b1 = __ldg(&m->b1[nt * 8 + 2 * t + 1]);
      acc[mt][nt][0] = b0; acc[mt][nt][1] = b1; acc[mt][nt][2] = b0; acc[mt][nt][3] = b1;
    }
  // layer 1: [32 x 32] x W1^T
#pragma unroll
  for (int ks = 0; ks < 2; ++ks) {
    uint32_t a[2][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      const uint32_t* r0 = reinterpret_cast<const uint32_t*>(rows + (16 * mt + g) * MLP_ROW);
      const uint32_t* r8 = reinterpret_cast<const uint32_t*>(rows + (16 * mt + g + 8) * MLP_ROW);
      a[mt][0] = r0[8 * ks + t];
      a[mt][1] = r8[8 * ks + t];
      a[mt][2] = r0[8 * ks + 4 + t];
      a[mt][3] = r8[8 * ks + 4 + t];
    }
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const uint32_t* wrow = reinterpret_cast<const uint32_t*>(m->w1 + (nt * 8 + g) * 32);
      const uint32_t b[2] = {__ldg(wrow + 8 * ks + t), __ldg(wrow + 8 * ks + 4 + t)};
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) mma_bf16_16816(acc[mt][nt], a[mt], b);
    }
  }
  // tanh, then the accumulators become layer 2's A fragments
  uint32_t h[2][2][4];  // [m-tile][k-step][frag]
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int ks = 0; ks < 2; ++ks) {
      const float* lo = acc[mt][2 * ks];
      const float* hi = acc[mt][2 * ks + 1];
      h[mt][ks][0] = pack_bf16(tanh_hw(lo[0]), tanh_hw(lo[1]));
      h[mt][ks][1] = pack_bf16(tanh_hw(lo[2]), tanh_hw(lo[3]));
      h[mt][ks][2] = pack_bf16(tanh_hw(hi[0]), tanh_hw(hi[1]));
      h[mt][ks][3] = pack_bf16(tanh_hw(hi[2]), tanh_hw(hi[3]));
    }
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const float b0 = __ldg(&m->b2[nt * 8 + 2 * t]), b1 = __ldg(&m->b2[nt * 8 + 2 * t + 1]);
      acc[mt][nt][0] = b0; acc[mt][nt][1] = b1; acc[mt][nt][2] = b0; acc[mt][nt][3] = b1;
    }
#pragma unroll
  for (int ks = 0; ks < 2; ++ks)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const uint32_t* wrow = reinterpret_cast<const uint32_t*>(m->w2 + (nt * 8 + g) * 32);
      const uint32_t b[2] = {__ldg(wrow + 8 * ks + t), __ldg(wrow + 8 * ks + 4 + t)};
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) mma_bf16_16816(acc[mt][nt], h[mt][ks], b);
    }
  // output layer: y = w3 . tanh(h2) + b3, reduced over the 4 lanes of a quad
  float y[2][2];  // [m-tile][row g / g+8]
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
    float s0 = 0.0f, s8 = 0.0f;
#pragma unroll
    for (int nt = 0; nt < 4; ++nt) {
      const float w0 = __ldg(&m->w3[nt * 8 + 2 * t]), w1 = __ldg(&m->w3[nt * 8 + 2 * t + 1]);
      s0 = fmaf(w0, tanh_hw(acc[mt][nt][0]), s0);
      s0 = fmaf(w1, tanh_hw(acc[mt][nt][1]), s0);
      s8 = fmaf(w0, tanh_hw(acc[mt][nt][2]), s8);
      s8 = fmaf(w1, tanh_hw(acc[mt][nt][3]), s8);
    }
    s0 += __shfl_xor_sync(0xffffffffu, s0, 1);
    s0 += __shfl_xor_sync(0xffffffffu, s0, 2);
    s8 += __shfl_xor_sync(0xffffffffu, s8, 1);
    s8 += __shfl_xor_sync(0xffffffffu, s8, 2);
    y[mt][0] = s0;
    y[mt][1] = s8;
  }
  if (t == 0) {
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {
      ysh[16 * mt + g] = y[mt][0];
      ysh[16 * mt + g + 8] = y[mt][1];
    }
  }
  __syncwarp();
  const float out = m->out_scale * (ysh[lane] + m->b3);
  __syncwarp();
  return out;
}

// Block-level entry: every thread of the (128-thread) block calls it with its
// node's features; returns the guess minus 2 for that node.
template <int Q>
__device__ __forceinline__ float mlp_guess_block(const MlpDev* __restrict__ m, const float x[Q]) {
  __shared__ __align__(16) __nv_bfloat16 rows[4][32 * MLP_ROW];
  __shared__ float ysh[4][32];
  const int w = threadIdx.x >> 5;
  return mlp_guess_warp<Q>(m, x, rows[w], ysh[w]);
}

}  // namespace mlbm
