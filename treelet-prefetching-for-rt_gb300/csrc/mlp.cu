// The learned treelet predictor: forward, softmax cross-entropy, backward,
// Adam and top-4, all on the GPU.
//
//   x  = [origin(3), dir(3), E[current](16)]           22 inputs (padded to 32)
//   h1 = GELU(x W1 + b1)                                64
//   h2 = GELU(h1 W2 + b2)                               64
//   z  = h2 W3 + b3                                     one logit per treelet
//
// Weights are used in BF16 with FP32 accumulation; FP32 master copies are
// what Adam updates.  The output layer, whose products span every treelet,
// runs on the fifth-generation tensor cores (tcgen05.mma with accumulators in
// tensor memory) fused with the softmax cross-entropy, so the batch x
// treelets logits are never stored (mlp_tc.cuh).  The two hidden layers
// (4096 x 64 x 64 at most) run on mma.sync m16n8k16 tiles.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "capi_internal.h"
#include "mlp_tc.cuh"

namespace {

constexpr int H = RT_MLP_HIDDEN;  // 64
constexpr int EMB = RT_MLP_EMBED; // 16
constexpr int XIN = 22;           // real inputs
constexpr int XP = 32;            // padded input width
using bf16 = __nv_bfloat16;

// ----------------------------------------------------------------- GEMM
// C[M x N] (+)= A[M x K] * B[K x N].  A is read row-major (AT = false:
// A[m * lda + k]) or transposed (AT = true: A[k * lda + m]); B is read
// row-major (BT = false: B[k * ldb + n]) or transposed (BT = true:
// B[n * ldb + k]).  64 x 64 CTA tile, 4 warps of 32 x 32, K in steps of 32;
// gridDim.z splits K, partial sums are added atomically (EPI_ACC).
enum Epi { EPI_STORE = 0, EPI_ACC = 1, EPI_BIAS_GELU = 2, EPI_BIAS = 3 };

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.0f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x) {
  const float cdf = 0.5f * (1.0f + erff(x * 0.70710678118654752f));
  const float pdf = 0.3989422804014327f * expf(-0.5f * x * x);
  return cdf + x * pdf;
}

template <bool AT, bool BT, int EPI>
__global__ void __launch_bounds__(128) gemm_kernel(int M, int N, int K, const bf16* __restrict__ A, int lda,
                                                   const bf16* __restrict__ B, int ldb, float* __restrict__ C,
                                                   int ldc, const float* __restrict__ bias, bf16* __restrict__ Hout) {
  constexpr int BM = 64, BN = 64, BK = 32, PAD = 8;
  __shared__ __align__(16) bf16 As[BM][BK + PAD];
  __shared__ __align__(16) bf16 Bs[BN][BK + PAD];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  // K range of this split
  const int splits = gridDim.z;
  const int kchunk = ((K + splits * BK - 1) / (splits * BK)) * BK;
  const int kbeg = blockIdx.z * kchunk, kend = min(K, kbeg + kchunk);
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.0f;
  const bf16 zero = __float2bfloat16(0.0f);
  for (int k0 = kbeg; k0 < kend; k0 += BK) {
    for (int e = tid; e < BM * BK; e += 128) {
      const int r = e / BK, c = e % BK;
      const int m = m0 + r, k = k0 + c;
      bf16 v = zero;
      if (m < M && k < kend) v = AT ? A[(size_t)k * lda + m] : A[(size_t)m * lda + k];
      As[r][c] = v;
    }
    for (int e = tid; e < BN * BK; e += 128) {
      const int r = e / BK, c = e % BK;
      const int n = n0 + r, k = k0 + c;
      bf16 v = zero;
      if (n < N && k < kend) v = BT ? B[(size_t)n * ldb + k] : B[(size_t)k * ldb + n];
      Bs[r][c] = v;
    }
    __syncthreads();
    const int g = lane >> 2, t = lane & 3;
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int rb = wm + i * 16;
        af[i][0] = *reinterpret_cast<const uint32_t*>(&As[rb + g][kk + 2 * t]);
        af[i][1] = *reinterpret_cast<const uint32_t*>(&As[rb + g + 8][kk + 2 * t]);
        af[i][2] = *reinterpret_cast<const uint32_t*>(&As[rb + g][kk + 2 * t + 8]);
        af[i][3] = *reinterpret_cast<const uint32_t*>(&As[rb + g + 8][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int nb = wn + j * 8;
        bfr[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[nb + g][kk + 2 * t]);
        bfr[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[nb + g][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j)
          asm volatile(
              "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
              "{%0,%1,%2,%3};\n"
              : "+f"(acc[i][j][0]), "+f"(acc[i][j][1]), "+f"(acc[i][j][2]), "+f"(acc[i][j][3])
              : "r"(af[i][0]), "r"(af[i][1]), "r"(af[i][2]), "r"(af[i][3]), "r"(bfr[j][0]), "r"(bfr[j][1]));
    }
    __syncthreads();
  }
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const int m = m0 + wm + i * 16 + g + (r >= 2 ? 8 : 0);
        const int n = n0 + wn + j * 8 + 2 * t + (r & 1);
        if (m >= M || n >= N) continue;
        float v = acc[i][j][r];
        float* dst = C + (size_t)m * ldc + n;
        if (EPI == EPI_ACC) {
          atomicAdd(dst, v);
        } else if (EPI == EPI_STORE) {
          *dst = v;
        } else {
          v += bias[n];
          *dst = v;
          if (EPI == EPI_BIAS_GELU) Hout[(size_t)m * ldc + n] = __float2bfloat16(gelu(v));
        }
      }
}

template <bool AT, bool BT, int EPI>
void gemm(int M, int N, int K, const bf16* A, int lda, const bf16* B, int ldb, float* C, int ldc, const float* bias,
          bf16* Hout, int splits, cudaStream_t st) {
  dim3 grid((N + 63) / 64, (M + 63) / 64, splits);
  gemm_kernel<AT, BT, EPI><<<grid, 128, 0, st>>>(M, N, K, A, lda, B, ldb, C, ldc, bias, Hout);
}

// ------------------------------------------------------------ elementwise
// A sample whose current treelet is out of range gets a zero embedding.
__global__ void gather_inputs(const rt_mlp_sample* __restrict__ s, int n, const bf16* __restrict__ E, uint32_t C,
                              bf16* __restrict__ X) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * XP) return;
  const int b = i / XP, c = i % XP;
  float v = 0.0f;
  if (c < 3) v = s[b].origin[c];
  else if (c < 6) v = s[b].dir[c - 3];
  else if (c < XIN) {
    const uint32_t cur = s[b].current;
    X[i] = cur < C ? E[(size_t)cur * EMB + (c - 6)] : __float2bfloat16(0.0f);
    return;
  }
  X[i] = __float2bfloat16(v);
}

// dZ = dH * GELU'(Z) as BF16.
__global__ void gelu_back(const float* __restrict__ dH, const float* __restrict__ Z, bf16* __restrict__ dZ, int count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) dZ[i] = __float2bfloat16(dH[i] * gelu_grad(Z[i]));
}

// out[c] += sum_r X[r][c]: one block per 128 rows, one thread per column
// (out starts at zero).  One block over all rows took 0.22 ms for 4,096 x 64.
__global__ void col_sum(const bf16* __restrict__ X, int rows, int cols, float* __restrict__ out) {
  const int c = threadIdx.x;
  if (c >= cols) return;
  const int r0 = blockIdx.x * 128, r1 = min(rows, r0 + 128);
  float s = 0.0f;
  for (int r = r0; r < r1; ++r) s += __bfloat162float(X[(size_t)r * cols + c]);
  atomicAdd(out + c, s);
}

__global__ void embed_grad(const float* __restrict__ dX, const rt_mlp_sample* __restrict__ s, int n, uint32_t C,
                           float* __restrict__ gE) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * EMB) return;
  const int b = i / EMB, j = i % EMB;
  const uint32_t cur = s[b].current;
  if (cur < C) atomicAdd(gE + (size_t)cur * EMB + j, dX[(size_t)b * XP + 6 + j]);
}

__global__ void copy_rows(const float* __restrict__ src, int src_ld, float* __restrict__ dst, int rows, int cols) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < rows * cols) dst[i] = src[(size_t)(i / cols) * src_ld + (i % cols)];
}

__global__ void adam(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v, const float* __restrict__ g,
                     uint64_t n, float lr, float c1, float c2) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = 0.9f * m[i] + 0.1f * gi;
  const float vi = 0.999f * v[i] + 0.001f * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + 1e-8f);
}

__global__ void to_bf16(const float* __restrict__ src, bf16* __restrict__ dst, uint64_t n) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = __float2bfloat16(src[i]);
}

// W1 (22 x 64) -> padded BF16 (32 x 64, rows 22..31 zero)
__global__ void w1_to_bf16(const float* __restrict__ w1, bf16* __restrict__ dst) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < XP * H) dst[i] = __float2bfloat16(i < XIN * H ? w1[i] : 0.0f);
}

// Deterministic initial values from a hash of (seed, index).
__global__ void init_params(float* __restrict__ p, uint64_t n, uint64_t seed, uint64_t offW1, uint64_t offb1,
                            uint64_t offW2, uint64_t offb2, uint64_t offW3, uint64_t offb3) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t h = rti::pcg_hash((uint32_t)i ^ rti::pcg_hash((uint32_t)seed));
  h = rti::pcg_hash(h ^ (uint32_t)(i >> 32));
  const float u = ((float)(h >> 8) * (1.0f / 16777216.0f)) * 2.0f - 1.0f;  // [-1, 1)
  float v;
  if (i < offW1) v = 0.1f * u;                       // embedding
  else if (i < offb1) v = u * 0.2132f;               // W1: 1/sqrt(22)
  else if (i < offW2) v = 0.0f;
  else if (i < offb2) v = u * 0.125f;                // W2: 1/sqrt(64)
  else if (i < offW3) v = 0.0f;
  else if (i < offb3) v = u * 0.125f;                // W3
  else v = 0.0f;
  p[i] = v;
}

}  // namespace

struct rt_mlp {
  int device = 0;
  uint32_t C = 0;
  uint64_t n_params = 0, offW1 = 0, offb1 = 0, offW2 = 0, offb2 = 0, offW3 = 0, offb3 = 0;
  float *P = nullptr, *M = nullptr, *V = nullptr, *G = nullptr;
  bf16 *E16 = nullptr, *W1_16 = nullptr, *W2_16 = nullptr;
  bf16 *W3T = nullptr, *W3P = nullptr, *H2X = nullptr;  // output-layer operands (mlp_tc.cuh)
  uint32_t Cp = 0;                                     // treelets padded to the output chunk
  bf16 *X = nullptr, *H1 = nullptr, *H2 = nullptr, *dZ2 = nullptr, *dZ1 = nullptr;
  float *Z1 = nullptr, *Z2 = nullptr, *dH2 = nullptr, *dH1 = nullptr, *dX = nullptr, *dW1 = nullptr;
  float *lse = nullptr, *part = nullptr;
  uint32_t* tstatus = nullptr;                         // bit 0: a bounded wait of the output layer gave up
  float* loss = nullptr;
  uint64_t step = 0;
  cudaStream_t st = nullptr;
};

namespace {

rt_status cfail(cudaError_t e, const char* what) {
  return rti::fail(RT_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define MLP_CUDA(call)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return cfail(e_, #call);     \
  } while (0)

template <class T>
cudaError_t mk(T** p, size_t count) {
  return cudaMalloc((void**)p, sizeof(T) * (count ? count : 1));
}

unsigned blocks(uint64_t n, unsigned t = 256) { return (unsigned)((n + t - 1) / t); }

void refresh_bf16(rt_mlp* m) {
  to_bf16<<<blocks((uint64_t)m->C * EMB), 256, 0, m->st>>>(m->P, m->E16, (uint64_t)m->C * EMB);
  w1_to_bf16<<<blocks(XP * H), 256, 0, m->st>>>(m->P + m->offW1, m->W1_16);
  to_bf16<<<blocks(H * H), 256, 0, m->st>>>(m->P + m->offW2, m->W2_16, H * H);
  tcm::w3_operands_kernel<<<m->Cp / 32, 256, 0, m->st>>>(m->P + m->offW3, m->C, m->Cp, m->W3T,
                                                                          m->W3P);
}

// Column splits of the row-tile passes of the output layer: two waves of
// two CTAs per SM over the row tiles of the batch (at most 152 splits: the
// partial-result buffer holds 2 x 152 per row).
uint32_t out_splits(const rt_mlp* m, uint32_t n) {
  const uint32_t tiles = (n + tcm::TM - 1) / tcm::TM, chunks = m->Cp / tcm::TN;
  const uint32_t want = (4 * 152 + tiles - 1) / tiles;
  return std::max<uint32_t>(1, std::min(std::min(chunks, want), 152u));
}

// Shared memory per CTA.  Pass 1 needs 49 KiB but asks for 80, so that
// exactly two CTAs share an SM (and its 512 TMEM columns).
constexpr size_t kSmemStats = 80 * 1024;
constexpr size_t kSmemDh2 = 16384 + 16384 + 32768 + 16384 + 512;
constexpr size_t kSmemDw3 = 16384 + 16384 + tcm::kDztBytes + 20480 + 512;

tcm::OutArgs out_args(rt_mlp* m, const rt_mlp_sample* s, uint32_t n) {
  tcm::OutArgs a{};
  a.h2 = m->H2;
  a.h2x = m->H2X;
  a.ldx = RT_MLP_MAX_BATCH;
  a.w3t = m->W3T;
  a.w3p = m->W3P;
  a.b3 = m->P + m->offb3;
  a.s = s;
  a.n = n;
  a.C = m->C;
  a.cp = m->Cp;
  a.splits = out_splits(m, n);
  a.part = m->part;
  a.lse = m->lse;
  a.dh2 = m->dH2;
  a.dw3 = m->G + m->offW3;
  a.db3 = m->G + m->offb3;
  a.status = m->tstatus;
  return a;
}

// Loss (and lse per row) of the output layer for n samples, or with top4 set
// the four largest logits of each sample instead.
void output_forward(rt_mlp* m, const rt_mlp_sample* s, uint32_t n, uint32_t* top4) {
  const tcm::OutArgs a = out_args(m, s, n);
  const dim3 grid((n + tcm::TM - 1) / tcm::TM, a.splits);
  if (top4) {
    tcm::out_stats_kernel<true><<<grid, tcm::kThreads, kSmemStats, m->st>>>(a);
    tcm::out_top4_kernel<<<blocks(n), 256, 0, m->st>>>(m->part, 2 * a.splits, n, top4);
    return;
  }
  tcm::out_stats_kernel<false><<<grid, tcm::kThreads, kSmemStats, m->st>>>(a);
  tcm::out_lse_kernel<<<blocks(n), 256, 0, m->st>>>(m->part, 2 * a.splits, n, s, m->C, m->lse, m->loss);
}

// Gradients of the output layer: dW3, db3 into G, dH2 (zeroed first).
void output_backward(rt_mlp* m, const rt_mlp_sample* s, uint32_t n) {
  const tcm::OutArgs a = out_args(m, s, n);
  tcm::h2x_kernel<<<blocks((uint64_t)tcm::HX * RT_MLP_MAX_BATCH), 256, 0, m->st>>>(m->H2, n, RT_MLP_MAX_BATCH,
                                                                                   m->H2X);
  tcm::out_dh2_kernel<<<dim3((n + tcm::TM - 1) / tcm::TM, a.splits), tcm::kThreads, kSmemDh2, m->st>>>(a);
  // two row halves per chunk, added into the zeroed gradient: 1,494 CTAs
  // (4.9 waves of 304) instead of 747 (2.5 waves)
  tcm::out_dw3_kernel<<<dim3(m->Cp / tcm::TN, 2), tcm::kThreads, kSmemDw3, m->st>>>(a);
}

int ksplit(int K, int tiles) {
  // enough CTAs to cover the GPU when the output has few tiles
  int s = 1;
  while (tiles * s < 304 && K / (s * 2) >= 256) s *= 2;
  return s;
}

// Forward (and, when grads is true, backward into G) for n samples.
rt_status run(rt_mlp* m, const rt_mlp_sample* s, uint32_t n, bool grads, uint32_t* top4) {
  const int B = (int)n;
  cudaStream_t st = m->st;
  gather_inputs<<<blocks((uint64_t)B * XP), 256, 0, st>>>(s, B, m->E16, m->C, m->X);
  gemm<false, false, EPI_BIAS_GELU>(B, H, XP, m->X, XP, m->W1_16, H, m->Z1, H, m->P + m->offb1, m->H1, 1, st);
  gemm<false, false, EPI_BIAS_GELU>(B, H, H, m->H1, H, m->W2_16, H, m->Z2, H, m->P + m->offb2, m->H2, 1, st);
  if (top4) {
    output_forward(m, s, n, top4);
    return RT_OK;
  }
  MLP_CUDA(cudaMemsetAsync(m->loss, 0, sizeof(float), st));
  output_forward(m, s, n, nullptr);
  if (!grads) return RT_OK;
  MLP_CUDA(cudaMemsetAsync(m->G, 0, sizeof(float) * m->n_params, st));
  // W3, b3 and dH2 = dz W3^T, on the tensor cores without the logits
  MLP_CUDA(cudaMemsetAsync(m->dH2, 0, sizeof(float) * B * H, st));
  output_backward(m, s, n);
  gelu_back<<<blocks((uint64_t)B * H), 256, 0, st>>>(m->dH2, m->Z2, m->dZ2, B * H);
  // W2, b2
  gemm<true, false, EPI_ACC>(H, H, B, m->H1, H, m->dZ2, H, m->G + m->offW2, H, nullptr, nullptr, ksplit(B, 1), st);
  col_sum<<<(B + 127) / 128, H, 0, st>>>(m->dZ2, B, H, m->G + m->offb2);
  // dH1 = dZ2 W2^T
  MLP_CUDA(cudaMemsetAsync(m->dH1, 0, sizeof(float) * B * H, st));
  gemm<false, true, EPI_ACC>(B, H, H, m->dZ2, H, m->W2_16, H, m->dH1, H, nullptr, nullptr, 1, st);
  gelu_back<<<blocks((uint64_t)B * H), 256, 0, st>>>(m->dH1, m->Z1, m->dZ1, B * H);
  // W1 (first 22 rows of the padded product), b1
  MLP_CUDA(cudaMemsetAsync(m->dW1, 0, sizeof(float) * XP * H, st));
  gemm<true, false, EPI_ACC>(XP, H, B, m->X, XP, m->dZ1, H, m->dW1, H, nullptr, nullptr, ksplit(B, 1), st);
  copy_rows<<<blocks(XIN * H), 256, 0, st>>>(m->dW1, H, m->G + m->offW1, XIN, H);
  col_sum<<<(B + 127) / 128, H, 0, st>>>(m->dZ1, B, H, m->G + m->offb1);
  // dX = dZ1 W1^T -> embedding rows
  MLP_CUDA(cudaMemsetAsync(m->dX, 0, sizeof(float) * B * XP, st));
  gemm<false, true, EPI_ACC>(B, XP, H, m->dZ1, H, m->W1_16, H, m->dX, XP, nullptr, nullptr, 1, st);
  embed_grad<<<blocks((uint64_t)B * EMB), 256, 0, st>>>(m->dX, s, B, m->C, m->G);
  return RT_OK;
}

// After the stream has been synchronised: RT_ERR_TIMEOUT (and the flag
// cleared) if a bounded wait of the output layer gave up.
rt_status check_status(rt_mlp* m, const char* who) {
  uint32_t st = 0;
  MLP_CUDA(cudaMemcpy(&st, m->tstatus, sizeof(st), cudaMemcpyDeviceToHost));
  if (st == 0) return RT_OK;
  MLP_CUDA(cudaMemset(m->tstatus, 0, sizeof(uint32_t)));
  return rti::fail(RT_ERR_TIMEOUT, std::string(who) + ": a bounded tensor-core wait gave up; results are invalid");
}

}  // namespace

extern "C" {

rt_status rt_mlp_create(rt_ctx* ctx, uint32_t n_treelets, uint64_t seed, rt_mlp** out) {
  if (!ctx || !out || n_treelets == 0) return rti::fail(RT_ERR_INVALID, "rt_mlp_create: bad argument");
  if (n_treelets > (1u << 24)) return rti::fail(RT_ERR_TOO_LARGE, "rt_mlp_create: at most 16M treelets");
  *out = nullptr;
  MLP_CUDA(cudaSetDevice(ctx->device));
  auto* m = new rt_mlp();
  m->device = ctx->device;
  const uint64_t C = n_treelets;
  m->C = n_treelets;
  m->offW1 = C * EMB;
  m->offb1 = m->offW1 + XIN * H;
  m->offW2 = m->offb1 + H;
  m->offb2 = m->offW2 + H * H;
  m->offW3 = m->offb2 + H;
  m->offb3 = m->offW3 + H * C;
  m->n_params = m->offb3 + C;
  const size_t MB = RT_MLP_MAX_BATCH;
  cudaError_t e = cudaSuccess;
  auto chk = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
  };
  chk(mk(&m->P, m->n_params));
  chk(mk(&m->M, m->n_params));
  chk(mk(&m->V, m->n_params));
  chk(mk(&m->G, m->n_params));
  chk(mk(&m->E16, C * EMB));
  chk(mk(&m->W1_16, XP * H));
  chk(mk(&m->W2_16, H * H));
  m->Cp = (uint32_t)((C + tcm::TN - 1) / tcm::TN * tcm::TN);
  chk(mk(&m->W3T, (size_t)m->Cp * H));
  chk(mk(&m->W3P, (size_t)m->Cp * H));
  chk(mk(&m->H2X, (size_t)tcm::HX * MB));
  chk(mk(&m->X, MB * XP));
  chk(mk(&m->H1, MB * H));
  chk(mk(&m->H2, MB * H));
  chk(mk(&m->dZ2, MB * H));
  chk(mk(&m->dZ1, MB * H));
  chk(mk(&m->Z1, MB * H));
  chk(mk(&m->Z2, MB * H));
  chk(mk(&m->lse, MB));
  chk(mk(&m->part, 8 * 152 * 2 * MB));  // 2 x 152 partial results of 8 floats per row
  chk(mk(&m->tstatus, 1));
  chk(mk(&m->dH2, MB * H));
  chk(mk(&m->dH1, MB * H));
  chk(mk(&m->dX, MB * XP));
  chk(mk(&m->dW1, XP * H));
  chk(mk(&m->loss, 1));
  chk(cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking));
  chk(cudaFuncSetAttribute(tcm::out_stats_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemStats));
  chk(cudaFuncSetAttribute(tcm::out_stats_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemStats));
  chk(cudaFuncSetAttribute(tcm::out_dh2_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemDh2));
  chk(cudaFuncSetAttribute(tcm::out_dw3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemDw3));
  if (e == cudaSuccess) e = cudaMemset(m->tstatus, 0, sizeof(uint32_t));
  if (e != cudaSuccess) {
    rt_mlp_destroy(m);
    return rti::fail(RT_ERR_OOM, std::string("rt_mlp_create: ") + cudaGetErrorString(e));
  }
  init_params<<<blocks(m->n_params), 256, 0, m->st>>>(m->P, m->n_params, seed, m->offW1, m->offb1, m->offW2,
                                                         m->offb2, m->offW3, m->offb3);
  cudaMemsetAsync(m->M, 0, sizeof(float) * m->n_params, m->st);
  cudaMemsetAsync(m->V, 0, sizeof(float) * m->n_params, m->st);
  refresh_bf16(m);
  e = cudaStreamSynchronize(m->st);
  if (e != cudaSuccess) {
    rt_mlp_destroy(m);
    return cfail(e, "rt_mlp_create");
  }
  *out = m;
  return RT_OK;
}

rt_status rt_mlp_destroy(rt_mlp* m) {
  if (!m) return RT_OK;
  cudaSetDevice(m->device);
  void* ptrs[] = {m->P, m->M, m->V, m->G, m->E16, m->W1_16, m->W2_16, m->W3T, m->W3P, m->H2X, m->X, m->H1,
                  m->H2, m->dZ2, m->dZ1, m->Z1, m->Z2, m->dH2, m->dH1, m->dX, m->dW1, m->lse, m->part,
                  m->tstatus, m->loss};
  for (void* p : ptrs) cudaFree(p);
  if (m->st) cudaStreamDestroy(m->st);
  delete m;
  return RT_OK;
}

rt_status rt_mlp_num_params(const rt_mlp* m, uint64_t* n) {
  if (!m || !n) return rti::fail(RT_ERR_INVALID, "rt_mlp_num_params: NULL");
  *n = m->n_params;
  return RT_OK;
}

rt_status rt_mlp_get_params(const rt_mlp* m, float* host) {
  if (!m || !host) return rti::fail(RT_ERR_INVALID, "rt_mlp_get_params: NULL");
  MLP_CUDA(cudaSetDevice(m->device));
  MLP_CUDA(cudaStreamSynchronize(m->st));
  MLP_CUDA(cudaMemcpy(host, m->P, sizeof(float) * m->n_params, cudaMemcpyDeviceToHost));
  return RT_OK;
}

rt_status rt_mlp_set_params(rt_mlp* m, const float* host) {
  if (!m || !host) return rti::fail(RT_ERR_INVALID, "rt_mlp_set_params: NULL");
  MLP_CUDA(cudaSetDevice(m->device));
  MLP_CUDA(cudaStreamSynchronize(m->st));
  MLP_CUDA(cudaMemcpy(m->P, host, sizeof(float) * m->n_params, cudaMemcpyHostToDevice));
  refresh_bf16(m);
  MLP_CUDA(cudaStreamSynchronize(m->st));
  return RT_OK;
}

rt_status rt_mlp_loss_grad(rt_mlp* m, const rt_mlp_sample* s, uint32_t n, float* loss, float* grads_host) {
  if (!m || !s || n == 0) return rti::fail(RT_ERR_INVALID, "rt_mlp_loss_grad: bad argument");
  if (n > RT_MLP_MAX_BATCH) return rti::fail(RT_ERR_TOO_LARGE, "rt_mlp_loss_grad: batch above RT_MLP_MAX_BATCH");
  MLP_CUDA(cudaSetDevice(m->device));
  rt_status st = run(m, s, n, grads_host != nullptr, nullptr);
  if (st != RT_OK) return st;
  MLP_CUDA(cudaGetLastError());
  MLP_CUDA(cudaStreamSynchronize(m->st));
  st = check_status(m, "rt_mlp_loss_grad");
  if (st != RT_OK) return st;
  if (loss) MLP_CUDA(cudaMemcpy(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost));
  if (grads_host) MLP_CUDA(cudaMemcpy(grads_host, m->G, sizeof(float) * m->n_params, cudaMemcpyDeviceToHost));
  return RT_OK;
}

rt_status rt_mlp_train_step(rt_mlp* m, const rt_mlp_sample* s, uint32_t n, float lr, float* loss) {
  if (!m || !s || n == 0) return rti::fail(RT_ERR_INVALID, "rt_mlp_train_step: bad argument");
  if (n > RT_MLP_MAX_BATCH) return rti::fail(RT_ERR_TOO_LARGE, "rt_mlp_train_step: batch above RT_MLP_MAX_BATCH");
  MLP_CUDA(cudaSetDevice(m->device));
  rt_status st = run(m, s, n, true, nullptr);
  if (st != RT_OK) return st;
  m->step += 1;
  const float c1 = 1.0f - powf(0.9f, (float)m->step), c2 = 1.0f - powf(0.999f, (float)m->step);
  adam<<<blocks(m->n_params), 256, 0, m->st>>>(m->P, m->M, m->V, m->G, m->n_params, lr, c1, c2);
  refresh_bf16(m);
  MLP_CUDA(cudaGetLastError());
  if (loss) {
    MLP_CUDA(cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->st));
    MLP_CUDA(cudaStreamSynchronize(m->st));
    return check_status(m, "rt_mlp_train_step");
  }
  return RT_OK;
}

rt_status rt_mlp_topk(rt_mlp* m, const rt_mlp_sample* s, uint32_t n, uint32_t* top4) {
  if (!m || !s || !top4) return rti::fail(RT_ERR_INVALID, "rt_mlp_topk: NULL");
  MLP_CUDA(cudaSetDevice(m->device));
  for (uint32_t b0 = 0; b0 < n; b0 += RT_MLP_MAX_BATCH) {
    const uint32_t nb = std::min<uint32_t>(RT_MLP_MAX_BATCH, n - b0);
    rt_status st = run(m, s + b0, nb, false, top4 + (size_t)b0 * 4);
    if (st != RT_OK) return st;
  }
  MLP_CUDA(cudaGetLastError());
  MLP_CUDA(cudaStreamSynchronize(m->st));
  return check_status(m, "rt_mlp_topk");
}

}  // extern "C"
