// mlp.cuh -- the learned branching scorer shared by the search kernel, the
// incumbent proposal and the batch inference entry point.
//
// Network: 16 features per candidate -> 128 -> 128 -> 1 logit, ReLU between
// layers.  Inference runs on the tensor cores with BF16 weights and
// activations and FP32 accumulation: one warp scores 16 candidates (one
// m16 row tile) with mma.sync.m16n8k16 (152 instructions per tile).  The
// FP32 master weights are trained by the hand-written kernels in mlp.cu.
//
// The scorer has no counterpart in the reference: it only changes which
// branching vertex u* is taken among candidates that the reference's rule
// (selectUstar, src/helpers.cc:1104-1168) would also accept, and proposes
// incumbents that the integer method verifies, so every pruning rule and the
// optimality proof stay the plain integer method.
//
// Packed weight layout (u32 words holding two bf16, lower index in the low
// half), in mma.sync B-fragment order so a lane loads its two words of a
// tile with one 8-byte load:
//   w1: tile nt (0..15)            -> [nt][lane] uint2   k rows 0..15
//   w2: tile (kc, nt) (8 x 16)     -> [kc][nt][lane] uint2
//   w3: tile kc (0..7), n padded to 8 (column 0 is the logit) -> [kc][lane]
// For tile (kc, nt), lane (g = lane / 4, t = lane % 4) holds
//   .x = W[16kc + 2t][8nt + g], W[16kc + 2t + 1][8nt + g]
//   .y = W[16kc + 2t + 8][8nt + g], W[16kc + 2t + 9][8nt + g]
// with W[in][out] the layer's weight matrix.
#pragma once
#include <cstdint>

#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace scs {

constexpr int MLP_IN = 16;
constexpr int MLP_H = 128;
constexpr int MLP_TILE = 16;  // candidates per warp evaluation
// parameter counts of the FP32 master copy, in file order:
// W1[16][128], b1[128], W2[128][128], b2[128], W3[128], b3
constexpr int MLP_NPARAM = MLP_IN * MLP_H + MLP_H + MLP_H * MLP_H + MLP_H + MLP_H + 1;
constexpr int MLP_W1_U2 = 16 * 32;      // uint2 per packed layer
constexpr int MLP_W2_U2 = 8 * 16 * 32;
constexpr int MLP_W3_U2 = 8 * 32;
constexpr int MLP_PACK_U2 = MLP_W1_U2 + MLP_W2_U2 + MLP_W3_U2;

struct MlpDev {
  const uint2 *w;      // packed w1 | w2 | w3 (MLP_PACK_U2 uint2)
  const float *bias;   // b1[128] | b2[128] | b3
};

// Host: the FP32 master parameters (file order) -> packed BF16 fragments
// (2 * MLP_PACK_U2 words) and the bias block (2 * MLP_H + 4 floats).
// Rounding is to nearest even, as __floats2bfloat162_rn on the device.
void mlp_pack(const float *params, std::vector<uint32_t> &packed, std::vector<float> &bias);

__device__ __forceinline__ uint32_t pack_bf16x2(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4],
                                         uint2 b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
      "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b.x), "r"(b.y));
}

// Scores of 16 candidates.  Call with the whole warp.  x points at the
// candidates' features, row r at x[r * ld .. r * ld + 16) (shared or
// global memory, FP32).  Returns the logit of row (lane % 16) in every lane
// (lanes 16..31 repeat rows 0..15).
__device__ __forceinline__ float mlp_score16(const MlpDev &M, const float *x, int ld) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  uint32_t xa[4];
  xa[0] = pack_bf16x2(x[g * ld + 2 * t], x[g * ld + 2 * t + 1]);
  xa[1] = pack_bf16x2(x[(g + 8) * ld + 2 * t], x[(g + 8) * ld + 2 * t + 1]);
  xa[2] = pack_bf16x2(x[g * ld + 2 * t + 8], x[g * ld + 2 * t + 9]);
  xa[3] = pack_bf16x2(x[(g + 8) * ld + 2 * t + 8], x[(g + 8) * ld + 2 * t + 9]);
  const uint2 *w1 = M.w, *w2 = M.w + MLP_W1_U2, *w3 = w2 + MLP_W2_U2;
  const float *b1 = M.bias, *b2 = M.bias + MLP_H;
  // layer 1: tile nt gives hidden columns 8nt..8nt+7; tiles (2kc, 2kc+1)
  // together are exactly the A fragment of layer 2's k-chunk kc
  uint32_t h1[8][4];
#pragma unroll
  for (int kc = 0; kc < 8; kc++) {
#pragma unroll
    for (int half = 0; half < 2; half++) {
      const int nt = 2 * kc + half;
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      mma_bf16(d, xa, __ldg(w1 + nt * 32 + lane));
      const float2 bb = __ldg(reinterpret_cast<const float2 *>(b1 + 8 * nt + 2 * t));
      h1[kc][2 * half] = pack_bf16x2(fmaxf(d[0] + bb.x, 0.f), fmaxf(d[1] + bb.y, 0.f));
      h1[kc][2 * half + 1] = pack_bf16x2(fmaxf(d[2] + bb.x, 0.f), fmaxf(d[3] + bb.y, 0.f));
    }
  }
  // reorder into A-fragment register order: {row g k-lo, row g+8 k-lo,
  // row g k-hi, row g+8 k-hi}
  // layers 2 and 3, one layer-3 k-chunk (two layer-2 output tiles) at a time
  float o[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
  for (int jc = 0; jc < 8; jc++) {
    float d0[4] = {0.f, 0.f, 0.f, 0.f}, d1[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kc = 0; kc < 8; kc++) {
      const uint32_t a[4] = {h1[kc][0], h1[kc][1], h1[kc][2], h1[kc][3]};
      mma_bf16(d0, a, __ldg(w2 + (kc * 16 + 2 * jc) * 32 + lane));
      mma_bf16(d1, a, __ldg(w2 + (kc * 16 + 2 * jc + 1) * 32 + lane));
    }
    const float2 c0 = __ldg(reinterpret_cast<const float2 *>(b2 + 16 * jc + 2 * t));
    const float2 c1 = __ldg(reinterpret_cast<const float2 *>(b2 + 16 * jc + 8 + 2 * t));
    const uint32_t a3[4] = {
        pack_bf16x2(fmaxf(d0[0] + c0.x, 0.f), fmaxf(d0[1] + c0.y, 0.f)),
        pack_bf16x2(fmaxf(d0[2] + c0.x, 0.f), fmaxf(d0[3] + c0.y, 0.f)),
        pack_bf16x2(fmaxf(d1[0] + c1.x, 0.f), fmaxf(d1[1] + c1.y, 0.f)),
        pack_bf16x2(fmaxf(d1[2] + c1.x, 0.f), fmaxf(d1[3] + c1.y, 0.f))};
    mma_bf16(o, a3, __ldg(w3 + jc * 32 + lane));
  }
  // column 0 of the output tile: lane t == 0 holds rows g (o[0]) and g+8 (o[2])
  const float b3 = __ldg(M.bias + 2 * MLP_H);
  const int r = lane & 15;
  const float v_lo = __shfl_sync(0xffffffffu, o[0], (r & 7) * 4);
  const float v_hi = __shfl_sync(0xffffffffu, o[2], (r & 7) * 4);
  return (r < 8 ? v_lo : v_hi) + b3;
}

// ---- candidate features ----
// Everything a feature needs about one candidate v of a task (C, R) and
// about the task.  The same function serves the search step, the trace the
// exact solver emits for training and the incumbent proposal, so the network
// sees one definition everywhere.
struct FeatIn {
  uint32_t dC, dR;        // v's neighbours in C and in R (inside the task)
  uint32_t dist;          // hop distance from q (full graph)
  uint32_t core;          // core number of v in the full graph
  uint32_t deg;           // v's degree in the query's local graph
  float score, score_max; // the reference's ustar score of v, best in list
  uint32_t is_best;       // v is the reference rule's u*
};
struct FeatTask {
  uint32_t s, csize, n_local, l, h, kl, ub, ubd, dmax;
};

__host__ __device__ inline float lg1p(float x) { return logf(1.0f + x); }

__host__ __device__ inline void make_features(const FeatIn &c, const FeatTask &k,
                                              float *f) {
  const float h = (float)k.h, cs = (float)(k.csize ? k.csize : 1);
  const float ldm = lg1p((float)k.dmax);
  f[0] = (float)c.dC / cs;
  f[1] = lg1p((float)c.dC) / lg1p(h);
  f[2] = lg1p((float)c.dR) / ldm;
  f[3] = fminf(fmaxf(((float)c.dC + (float)c.dR - (float)k.kl) / h, -1.f), 4.f);
  f[4] = (float)c.dist / (float)(k.ubd + 1);
  f[5] = lg1p((float)c.core) / ldm;
  f[6] = fminf(fmaxf(((float)c.core - (float)k.kl) / h, -1.f), 4.f);
  f[7] = c.score_max > 0.f ? c.score / c.score_max : 0.f;
  f[8] = c.is_best ? 1.f : 0.f;
  f[9] = lg1p((float)c.deg) / ldm;
  f[10] = (float)k.csize / h;
  f[11] = (float)k.l / h;
  f[12] = (float)k.kl / h;
  f[13] = fminf(((float)k.ub - (float)k.kl) / h, 4.f);
  f[14] = (h - (float)k.csize) / h;
  f[15] = lg1p((float)k.s) / lg1p((float)(k.n_local ? k.n_local : 1));
}

}  // namespace scs
