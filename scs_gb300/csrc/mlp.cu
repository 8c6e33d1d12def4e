// mlp.cu -- training and batch inference of the learned branching scorer.
//
// Training (FP32, hand-written kernels): forward 16 -> 128 -> 128 -> 1 with
// ReLU, weighted binary cross-entropy on the logit, backward by the chain
// rule, Adam.  Every matrix product goes through one tiled kernel
// (64 x 64 output tile per 256-thread CTA, 16-deep K slices staged in shared
// memory, 4 x 4 outputs per thread) with a fused epilogue: bias + ReLU in the
// forward pass, the ReLU derivative mask in the backward pass.  Products are
// summed in a fixed order, so gradients are deterministic.
//
// Inference: the packed BF16 weights (mlp.cuh) and one warp per 16 rows on
// the tensor cores (mma.sync m16n8k16, FP32 accumulate) -- the same device
// code the search kernel runs inside its branching step.
//
// The network has no counterpart in the reference; see mlp.cuh.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "../../include/scs.h"
#include "mlp.cuh"

namespace scs {

// ---------------------------------------------------------------------------
// host: BF16 rounding and weight packing
// ---------------------------------------------------------------------------
static inline uint16_t bf16_rne(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7F800000u) == 0x7F800000u) return (uint16_t)(u >> 16);  // inf/nan
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

static inline uint32_t pack2(float lo, float hi) {
  return (uint32_t)bf16_rne(lo) | ((uint32_t)bf16_rne(hi) << 16);
}

// B fragments of an [in][out] matrix W (row stride ld_out) for the tile
// at rows 16kc.., columns 8nt..; columns at or beyond n_out are zero.
static void pack_tile(const float *W, int ld_out, int n_out, int kc, int nt,
                      uint32_t *dst /* 64 words */) {
  for (int lane = 0; lane < 32; lane++) {
    const int g = lane >> 2, t = lane & 3, col = 8 * nt + g;
    auto w = [&](int k) { return col < n_out ? W[(size_t)k * ld_out + col] : 0.f; };
    const int k0 = 16 * kc + 2 * t;
    dst[2 * lane] = pack2(w(k0), w(k0 + 1));
    dst[2 * lane + 1] = pack2(w(k0 + 8), w(k0 + 9));
  }
}

void mlp_pack(const float *P, std::vector<uint32_t> &packed, std::vector<float> &bias) {
  const float *W1 = P, *b1 = W1 + MLP_IN * MLP_H, *W2 = b1 + MLP_H, *b2 = W2 + MLP_H * MLP_H,
              *W3 = b2 + MLP_H, *b3 = W3 + MLP_H;
  packed.assign((size_t)MLP_PACK_U2 * 2, 0u);
  uint32_t *p = packed.data();
  for (int nt = 0; nt < 16; nt++, p += 64) pack_tile(W1, MLP_H, MLP_H, 0, nt, p);
  for (int kc = 0; kc < 8; kc++)
    for (int nt = 0; nt < 16; nt++, p += 64) pack_tile(W2, MLP_H, MLP_H, kc, nt, p);
  for (int kc = 0; kc < 8; kc++, p += 64) pack_tile(W3, 1, 1, kc, 0, p);
  bias.assign(2 * MLP_H + 4, 0.f);
  std::copy(b1, b1 + MLP_H, bias.begin());
  std::copy(b2, b2 + MLP_H, bias.begin() + MLP_H);
  bias[2 * MLP_H] = b3[0];
}

// ---------------------------------------------------------------------------
// device: tiled FP32 matrix product with fused epilogues
// ---------------------------------------------------------------------------
enum { EPI_STORE = 0, EPI_BIAS = 1, EPI_BIAS_RELU = 2, EPI_MASK = 3 };

// C[M x N] = op(A)[M x K] * op(B)[K x N], then the epilogue.
// op(A)(i, k) = TA ? A[k * lda + i] : A[i * lda + k]
// op(B)(k, j) = TB ? B[j * ldb + k] : B[k * ldb + j]
// EPI_BIAS(_RELU): + bias[j] (then max(., 0)); EPI_MASK: * (Mk[i*ldm+j] > 0)
template <bool TA, bool TB, int EPI>
__global__ void __launch_bounds__(256)
gemm_kernel(int M, int N, int K, const float *__restrict__ A, int lda,
            const float *__restrict__ B, int ldb, float *__restrict__ C, int ldc,
            const float *__restrict__ bias, const float *__restrict__ Mk, int ldm) {
  __shared__ float As[16][64 + 4];
  __shared__ float Bs[16][64 + 4];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int i0 = blockIdx.y * 64, j0 = blockIdx.x * 64;
  float acc[4][4] = {};
  for (int k0 = 0; k0 < K; k0 += 16) {
    for (int e = threadIdx.x; e < 16 * 64; e += 256) {
      const int kk = e >> 6, ii = e & 63;  // A tile: column kk, row ii
      const int gi = i0 + ii, gk = k0 + kk;
      float a = 0.f;
      if (gi < M && gk < K) a = TA ? A[(size_t)gk * lda + gi] : A[(size_t)gi * lda + gk];
      As[kk][ii] = a;
      const int jj = e & 63, gj = j0 + jj;
      float b = 0.f;
      if (gj < N && gk < K) b = TB ? B[(size_t)gj * ldb + gk] : B[(size_t)gk * ldb + gj];
      Bs[kk][jj] = b;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; kk++) {
      float a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; r++) a[r] = As[kk][ty + 16 * r];
#pragma unroll
      for (int c = 0; c < 4; c++) b[c] = Bs[kk][tx + 16 * c];
#pragma unroll
      for (int r = 0; r < 4; r++)
#pragma unroll
        for (int c = 0; c < 4; c++) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; r++) {
    const int i = i0 + ty + 16 * r;
    if (i >= M) continue;
#pragma unroll
    for (int c = 0; c < 4; c++) {
      const int j = j0 + tx + 16 * c;
      if (j >= N) continue;
      float v = acc[r][c];
      if (EPI == EPI_BIAS || EPI == EPI_BIAS_RELU) v += bias[j];
      if (EPI == EPI_BIAS_RELU) v = fmaxf(v, 0.f);
      if (EPI == EPI_MASK) v = Mk[(size_t)i * ldm + j] > 0.f ? v : 0.f;
      C[(size_t)i * ldc + j] = v;
    }
  }
}

template <bool TA, bool TB, int EPI>
static cudaError_t gemm(cudaStream_t st, int M, int N, int K, const float *A, int lda,
                        const float *B, int ldb, float *C, int ldc, const float *bias = nullptr,
                        const float *Mk = nullptr, int ldm = 0) {
  dim3 grid((N + 63) / 64, (M + 63) / 64);
  gemm_kernel<TA, TB, EPI><<<grid, 256, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, Mk, ldm);
  return cudaGetLastError();
}

// weighted BCE on logits: loss_i = w_i (softplus(z_i) - y_i z_i); dz_i =
// w_i (sigmoid(z_i) - y_i) / wsum.  loss accumulates sum_i loss_i / wsum.
__global__ void bce_kernel(int n, const float *z, const float *y, const float *w, float inv_wsum,
                           float *dz, double *loss) {
  __shared__ double red[8];
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float zi = z[i], yi = y[i], wi = w ? w[i] : 1.f;
    const float sp = zi > 0.f ? zi + log1pf(expf(-zi)) : log1pf(expf(zi));
    const float p = 1.f / (1.f + expf(-zi));
    acc += (double)wi * ((double)sp - (double)yi * (double)zi);
    dz[i] = wi * (p - yi) * inv_wsum;
  }
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += red[k];
    atomicAdd(loss, s * (double)inv_wsum);
  }
}

// out[j] = sum_i X[i * ld + j], i < n (one thread per column, fixed order)
__global__ void colsum_kernel(int n, int cols, const float *X, int ld, float *out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= cols) return;
  float s = 0.f;
  for (int i = 0; i < n; i++) s += X[(size_t)i * ld + j];
  out[j] = s;
}

__global__ void adam_kernel(int n, float *p, const float *g, float *m, float *v, float lr,
                            float b1, float b2, float eps, float wd, float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i] + wd * p[i];
  const float mi = b1 * m[i] + (1.f - b1) * gi;
  const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// gather rows idx[0..n) of X (16 wide), y, w into a batch
__global__ void gather_kernel(int n, const uint32_t *idx, const float *X, const float *y,
                              const float *w, float *bx, float *by, float *bw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * MLP_IN) return;
  const int r = i / MLP_IN, c = i % MLP_IN;
  const uint32_t s = idx[r];
  bx[i] = X[(size_t)s * MLP_IN + c];
  if (c == 0) {
    by[r] = y[s];
    bw[r] = w ? w[s] : 1.f;
  }
}

// batch inference: one warp per 16 rows of X (rows padded with zeros)
__global__ void mlp_infer_kernel(MlpDev M, const float *X, int n_tiles, float *out) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (warp >= n_tiles) return;
  const float z = mlp_score16(M, X + (size_t)warp * MLP_TILE * MLP_IN, MLP_IN);
  const int lane = threadIdx.x & 31;
  if (lane < 16) out[warp * MLP_TILE + lane] = z;
}

// Device buffers of one training/gradient run.
struct MlpRun {
  int cap = 0;
  float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  float *x = nullptr, *y = nullptr, *w = nullptr;
  float *h1 = nullptr, *h2 = nullptr, *z = nullptr, *dz = nullptr, *d2 = nullptr, *d1 = nullptr;
  double *loss = nullptr;
  std::vector<void *> all;
  cudaError_t alloc(int batch) {
    cap = batch;
    auto A = [&](auto **ptr, size_t count) {
      cudaError_t e = cudaMalloc((void **)ptr, std::max<size_t>(count, 1) * sizeof(**ptr));
      if (e == cudaSuccess) all.push_back(*ptr);
      return e;
    };
    cudaError_t e;
    if ((e = A(&p, MLP_NPARAM)) || (e = A(&g, MLP_NPARAM)) || (e = A(&m, MLP_NPARAM)) ||
        (e = A(&v, MLP_NPARAM)) || (e = A(&x, (size_t)batch * MLP_IN)) || (e = A(&y, batch)) ||
        (e = A(&w, batch)) || (e = A(&h1, (size_t)batch * MLP_H)) ||
        (e = A(&h2, (size_t)batch * MLP_H)) || (e = A(&z, batch)) || (e = A(&dz, batch)) ||
        (e = A(&d2, (size_t)batch * MLP_H)) || (e = A(&d1, (size_t)batch * MLP_H)) ||
        (e = A(&loss, 1)))
      return e;
    return cudaSuccess;
  }
  ~MlpRun() {
    for (void *q : all) cudaFree(q);
  }
};

// Offsets of the parameter blocks in the flat vector (file order).
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + MLP_IN * MLP_H, OFF_W2 = OFF_B1 + MLP_H,
              OFF_B2 = OFF_W2 + MLP_H * MLP_H, OFF_W3 = OFF_B2 + MLP_H, OFF_B3 = OFF_W3 + MLP_H;
static_assert(OFF_B3 + 1 == MLP_NPARAM, "parameter layout");

// Loss and gradient of the batch already in R.x / R.y / R.w (n rows) at
// parameters R.p; gradient into R.g, loss (weighted mean) into R.loss.
static cudaError_t mlp_loss_grad(MlpRun &R, int n, float wsum, cudaStream_t st) {
  cudaError_t e;
  const float *P = R.p;
  float *G = R.g;
  if ((e = cudaMemsetAsync(R.loss, 0, sizeof(double), st))) return e;
  // forward
  if ((e = gemm<false, false, EPI_BIAS_RELU>(st, n, MLP_H, MLP_IN, R.x, MLP_IN, P + OFF_W1, MLP_H,
                                             R.h1, MLP_H, P + OFF_B1)))
    return e;
  if ((e = gemm<false, false, EPI_BIAS_RELU>(st, n, MLP_H, MLP_H, R.h1, MLP_H, P + OFF_W2, MLP_H,
                                             R.h2, MLP_H, P + OFF_B2)))
    return e;
  if ((e = gemm<false, false, EPI_BIAS>(st, n, 1, MLP_H, R.h2, MLP_H, P + OFF_W3, 1, R.z, 1,
                                        P + OFF_B3)))
    return e;
  bce_kernel<<<std::min((n + 255) / 256, 1024), 256, 0, st>>>(n, R.z, R.y, R.w, 1.f / wsum, R.dz,
                                                              R.loss);
  if ((e = cudaGetLastError())) return e;
  // backward
  if ((e = gemm<true, false, EPI_STORE>(st, MLP_H, 1, n, R.h2, MLP_H, R.dz, 1, G + OFF_W3, 1)))
    return e;
  colsum_kernel<<<1, 32, 0, st>>>(n, 1, R.dz, 1, G + OFF_B3);
  if ((e = gemm<false, true, EPI_MASK>(st, n, MLP_H, 1, R.dz, 1, P + OFF_W3, 1, R.d2, MLP_H,
                                       nullptr, R.h2, MLP_H)))
    return e;
  if ((e = gemm<true, false, EPI_STORE>(st, MLP_H, MLP_H, n, R.h1, MLP_H, R.d2, MLP_H,
                                        G + OFF_W2, MLP_H)))
    return e;
  colsum_kernel<<<1, MLP_H, 0, st>>>(n, MLP_H, R.d2, MLP_H, G + OFF_B2);
  if ((e = gemm<false, true, EPI_MASK>(st, n, MLP_H, MLP_H, R.d2, MLP_H, P + OFF_W2, MLP_H, R.d1,
                                       MLP_H, nullptr, R.h1, MLP_H)))
    return e;
  if ((e = gemm<true, false, EPI_STORE>(st, MLP_IN, MLP_H, n, R.x, MLP_IN, R.d1, MLP_H,
                                        G + OFF_W1, MLP_H)))
    return e;
  colsum_kernel<<<1, MLP_H, 0, st>>>(n, MLP_H, R.d1, MLP_H, G + OFF_B1);
  return cudaGetLastError();
}

static std::string g_mlp_err;

static int fail(cudaError_t e, const char *what) {
  g_mlp_err = std::string(what) + ": " + cudaGetErrorString(e);
  return SCS_ECUDA;
}

}  // namespace scs

using namespace scs;

extern "C" {

const char *scs_mlp_last_error(void) { return g_mlp_err.c_str(); }

int scs_mlp_grad(const float *params, const float *X, const float *y, const float *w,
                 uint64_t n, double *loss, float *grad, int device) {
  if (!params || !X || !y || !loss || !grad || n == 0 || n > (1u << 24)) return SCS_EINVAL;
  cudaError_t e;
  if ((e = cudaSetDevice(device))) return fail(e, "cudaSetDevice");
  MlpRun R;
  if ((e = R.alloc((int)n))) return fail(e, "cudaMalloc");
  cudaStream_t st = nullptr;
  double wsum = 0.0;
  for (uint64_t i = 0; i < n; i++) wsum += w ? (double)w[i] : 1.0;
  if (wsum <= 0.0) return SCS_EINVAL;
  std::vector<float> ones;
  if (!w) ones.assign(n, 1.f);
  if ((e = cudaMemcpy(R.p, params, MLP_NPARAM * 4ull, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(R.x, X, n * MLP_IN * 4ull, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(R.y, y, n * 4ull, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(R.w, w ? w : ones.data(), n * 4ull, cudaMemcpyHostToDevice)))
    return fail(e, "copy in");
  if ((e = mlp_loss_grad(R, (int)n, (float)wsum, st))) return fail(e, "gradient kernels");
  if ((e = cudaMemcpy(grad, R.g, MLP_NPARAM * 4ull, cudaMemcpyDeviceToHost)) ||
      (e = cudaMemcpy(loss, R.loss, sizeof(double), cudaMemcpyDeviceToHost)))
    return fail(e, "copy out");
  return 0;
}

int scs_mlp_train(const float *X, const float *y, const float *w, uint64_t n,
                  const scs_mlp_train_cfg *cfg, float *params, float *epoch_loss, int device) {
  if (!X || !y || !cfg || !params || n == 0 || n > (1u << 26)) return SCS_EINVAL;
  const int batch = (int)std::min<uint64_t>(cfg->batch ? cfg->batch : 4096, n);
  const int epochs = cfg->epochs ? (int)cfg->epochs : 20;
  cudaError_t e;
  if ((e = cudaSetDevice(device))) return fail(e, "cudaSetDevice");
  MlpRun R;
  if ((e = R.alloc(batch))) return fail(e, "cudaMalloc");
  float *dX = nullptr, *dy = nullptr, *dw = nullptr;
  uint32_t *didx = nullptr;
  struct Frees {
    std::vector<void *> v;
    ~Frees() {
      for (void *p : v) cudaFree(p);
    }
  } fr;
  auto A = [&](auto **p, size_t bytes) {
    cudaError_t r = cudaMalloc((void **)p, bytes);
    if (r == cudaSuccess) fr.v.push_back(*p);
    return r;
  };
  if ((e = A(&dX, n * MLP_IN * 4ull)) || (e = A(&dy, n * 4ull)) || (e = A(&dw, n * 4ull)) ||
      (e = A(&didx, n * 4ull)))
    return fail(e, "cudaMalloc");
  std::vector<float> ones;
  if (!w) ones.assign(n, 1.f);
  if ((e = cudaMemcpy(dX, X, n * MLP_IN * 4ull, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(dy, y, n * 4ull, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(dw, w ? w : ones.data(), n * 4ull, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(R.p, params, MLP_NPARAM * 4ull, cudaMemcpyHostToDevice)) ||
      (e = cudaMemset(R.m, 0, MLP_NPARAM * 4ull)) || (e = cudaMemset(R.v, 0, MLP_NPARAM * 4ull)))
    return fail(e, "copy in");
  const float lr = cfg->lr > 0 ? cfg->lr : 1e-3f;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  std::mt19937_64 rng(cfg->seed);
  std::vector<uint32_t> perm(n), bw_host;
  for (uint64_t i = 0; i < n; i++) perm[i] = (uint32_t)i;
  std::vector<float> wh(w ? w : ones.data(), (w ? w : ones.data()) + n);
  long step = 0;
  for (int ep = 0; ep < epochs; ep++) {
    std::shuffle(perm.begin(), perm.end(), rng);
    if ((e = cudaMemcpy(didx, perm.data(), n * 4ull, cudaMemcpyHostToDevice)))
      return fail(e, "copy perm");
    double ep_loss = 0.0, ep_w = 0.0;
    for (uint64_t b0 = 0; b0 + batch <= n || (b0 < n && b0 == 0); b0 += batch) {
      const int nb = (int)std::min<uint64_t>(batch, n - b0);
      double wsum = 0.0;
      for (int i = 0; i < nb; i++) wsum += wh[perm[b0 + i]];
      if (wsum <= 0.0) continue;
      gather_kernel<<<(nb * MLP_IN + 255) / 256, 256>>>(nb, didx + b0, dX, dy, dw, R.x, R.y,
                                                        R.w);
      if ((e = cudaGetLastError())) return fail(e, "gather");
      if ((e = mlp_loss_grad(R, nb, (float)wsum, nullptr))) return fail(e, "gradient kernels");
      step++;
      const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
      adam_kernel<<<(MLP_NPARAM + 255) / 256, 256>>>(MLP_NPARAM, R.p, R.g, R.m, R.v, lr, b1, b2,
                                                     eps, cfg->weight_decay, c1, c2);
      if ((e = cudaGetLastError())) return fail(e, "adam");
      double l = 0.0;
      if ((e = cudaMemcpy(&l, R.loss, sizeof(double), cudaMemcpyDeviceToHost)))
        return fail(e, "loss");
      ep_loss += l * wsum;
      ep_w += wsum;
    }
    if (epoch_loss) epoch_loss[ep] = (float)(ep_w > 0 ? ep_loss / ep_w : 0.0);
  }
  if ((e = cudaMemcpy(params, R.p, MLP_NPARAM * 4ull, cudaMemcpyDeviceToHost)))
    return fail(e, "copy out");
  return 0;
}

int scs_mlp_infer(const float *params, const float *X, uint64_t n, float *out, int device) {
  if (!params || !X || !out || n == 0 || n > (1u << 26)) return SCS_EINVAL;
  cudaError_t e;
  if ((e = cudaSetDevice(device))) return fail(e, "cudaSetDevice");
  std::vector<uint32_t> packed;
  std::vector<float> bias;
  mlp_pack(params, packed, bias);
  const uint64_t tiles = (n + MLP_TILE - 1) / MLP_TILE;
  uint2 *dw = nullptr;
  float *db = nullptr, *dx = nullptr, *dout = nullptr;
  struct Frees {
    std::vector<void *> v;
    ~Frees() {
      for (void *p : v) cudaFree(p);
    }
  } fr;
  auto A = [&](auto **p, size_t bytes) {
    cudaError_t r = cudaMalloc((void **)p, bytes);
    if (r == cudaSuccess) fr.v.push_back(*p);
    return r;
  };
  if ((e = A(&dw, packed.size() * 4)) || (e = A(&db, bias.size() * 4)) ||
      (e = A(&dx, tiles * MLP_TILE * MLP_IN * 4)) || (e = A(&dout, tiles * MLP_TILE * 4)))
    return fail(e, "cudaMalloc");
  if ((e = cudaMemcpy(dw, packed.data(), packed.size() * 4, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(db, bias.data(), bias.size() * 4, cudaMemcpyHostToDevice)) ||
      (e = cudaMemset(dx, 0, tiles * MLP_TILE * MLP_IN * 4)) ||
      (e = cudaMemcpy(dx, X, n * MLP_IN * 4, cudaMemcpyHostToDevice)))
    return fail(e, "copy in");
  MlpDev M{dw, db};
  const int warps_per_block = 8;
  const unsigned blocks = (unsigned)((tiles + warps_per_block - 1) / warps_per_block);
  mlp_infer_kernel<<<blocks, 32 * warps_per_block>>>(M, dx, (int)tiles, dout);
  if ((e = cudaGetLastError())) return fail(e, "mlp_infer_kernel");
  if ((e = cudaMemcpy(out, dout, n * 4, cudaMemcpyDeviceToHost))) return fail(e, "copy out");
  return 0;
}

}  // extern "C"
