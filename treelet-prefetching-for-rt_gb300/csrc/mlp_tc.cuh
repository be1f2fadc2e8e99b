// The predictor's output layer on the fifth-generation tensor cores
// (tcgen05.mma, accumulators in tensor memory), fused with its softmax
// cross-entropy so that the batch x treelets logits never reach global memory.
//
//   z[b, c] = h2[b, :] . W3[:, c] + b3[c]            (K = 64, c over all treelets)
//   loss    = mean_b (logsumexp_c z[b, c] - z[b, target_b])
//   dz      = (softmax(z) - onehot(target)) / n
//   dW3 = h2^T dz,  db3 = column sums of dz,  dh2 = dz W3^T
//
// Three passes recompute the logits tile by tile instead of storing them:
//   out_stats_kernel  per (128-row tile, column split): the online max and
//                     exp-sum of every row, and the target's logit (or, for
//                     prediction, the four largest logits);
//   out_dh2_kernel    per (row tile, column split): dz for the tile, then
//                     dh2 += dz . W3 on the tensor cores, summed across
//                     splits with atomics;
//   out_dw3_kernel    per 128-column chunk and half of the row tiles: dz^T,
//                     then [dW3 | db3]^T += dz^T . [h2 | 1] on the tensor
//                     cores, added into the zeroed gradient.
//
// Operands live in shared memory in the canonical K-major layout without
// swizzle: 8-row x 16-byte core matrices, core matrices of one row group
// 128 bytes apart along K (the leading-dimension offset; 144 in the dW3
// pass's dz^T tile), row groups 16 * (K extent) bytes apart (the
// stride-dimension offset).  One thread issues
// the MMAs and commits them to an mbarrier; every wait is bounded and a wait
// that gives up sets the status word instead of hanging.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace tcm {

using bf16 = __nv_bfloat16;

constexpr int TM = 128;          // rows of a tile (TMEM lanes)
constexpr int TN = 128;          // columns (treelets) of a chunk
constexpr int HK = 64;           // hidden width (K of the logits product)
constexpr int HX = 80;           // [h2 | 1 | 0 ...] rows of the dW3 operand
// Eight warps a CTA: warp w reads TMEM lanes 32 (w % 4) .. 32 (w % 4) + 31
// (the lanes a warp may access) and column half w / 4 of every chunk.
constexpr int kThreads = 256;
// TMEM columns a CTA allocates: two CTAs share an SM's 512, so one CTA's
// epilogue runs while the other's MMAs and copies do.
constexpr uint32_t kTmemCols = 256;
constexpr uint32_t kTries = 1u << 22;
constexpr float kLog2e = 1.4426950408889634f;

// 2^x (MUFU ex2, flush-to-zero): the softmax exponentials in base 2.
__device__ __forceinline__ float ex2(float x) {
  float y;
  asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor: K-major, no swizzle, leading-dimension
// offset 128 bytes, the given stride-dimension offset, descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t addr, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)(128u >> 4) << 16) | ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) |
         ((uint64_t)1 << 46);
}

// Instruction descriptor of kind::f16: BF16 A and B (both K-major), FP32 accumulator.
__host__ __device__ constexpr uint32_t idesc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t id, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(id), "r"(accumulate));
}

__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
               : "memory");
}

__device__ __forceinline__ void bar_init(uint64_t* bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(su32(bar)));
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for the phase of the given parity; false if it gave up.
__device__ __forceinline__ bool bar_wait(uint64_t* bar, uint32_t parity) {
  for (uint32_t i = 0; i < kTries; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(su32(bar)), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// kTmemCols TMEM columns for the CTA (one warp allocates); returns the base address.
// The .sync.aligned tcgen05 instructions need their whole warp converged,
// hence the __syncwarp before each.
__device__ __forceinline__ uint32_t tmem_alloc(uint32_t* slot, int warp) {
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(slot)),
                 "n"(kTmemCols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  return *slot;
}

__device__ __forceinline__ void tmem_free(uint32_t base, int warp) {
  tc_before_sync();
  __syncthreads();
  __syncwarp();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "n"(kTmemCols));
}

// 32 consecutive FP32 columns of this thread's TMEM lane; every lane of the
// warp must call it (the load is warp-collective).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  __syncwarp();
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

// Byte offset of element (row r, k) of a K-major tile whose K extent is kx.
__device__ __forceinline__ uint32_t koff(uint32_t r, uint32_t k, uint32_t kx) {
  return (r >> 3) * (kx * 16u) + (k >> 3) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// Asynchronous 16-byte copy global -> shared (cp.async, L2 only).
__device__ __forceinline__ void cp16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(su32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(su32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Copies rows [r0, r0 + rows) x K columns [k0, k0 + kx) of a row-major BF16
// matrix (row stride ld elements, 16-byte aligned rows) into a K-major tile;
// rows past `valid` read as zero (written directly, not copied).
__device__ __forceinline__ void load_tile(uint8_t* tile, const bf16* g, uint64_t ld, uint32_t r0, uint32_t rows,
                                          uint32_t valid, uint32_t k0, uint32_t kx) {
  const uint32_t chunks = rows * (kx / 8u);
  for (uint32_t i = threadIdx.x; i < chunks; i += blockDim.x) {
    const uint32_t r = i / (kx / 8u), c = i % (kx / 8u);
    uint8_t* dst = tile + koff(r, c * 8u, kx);
    if (r0 + r < valid) cp16(dst, g + (uint64_t)(r0 + r) * ld + k0 + c * 8u);
    else *reinterpret_cast<uint4*>(dst) = make_uint4(0, 0, 0, 0);
  }
}

struct OutArgs {
  const bf16* h2;       // [n][64] hidden activations of the last layer
  const bf16* h2x;      // [80][ldx]: h2^T, then a row of ones for valid rows, zeros
  uint32_t ldx;         // row stride of h2x (elements)
  const bf16* w3t;      // [cp][64]: W3^T, rows past C zero
  const bf16* w3p;      // [64][cp]: W3, columns past C zero
  const float* b3;      // [C]
  const rt_mlp_sample* s;
  uint32_t n, C, cp;    // rows, treelets, padded treelets (multiple of TN)
  uint32_t splits;      // column splits of the row-tile passes
  float* part;          // [3][splits][n]: max, exp-sum, target logit (stats); or [splits][n][8] top-4 (pairs)
  const float* lse;     // [n]
  float* dh2;           // [n][64], summed atomically
  float* dw3;           // [64][C]
  float* db3;           // [C]
  uint32_t* status;     // bit 0: a bounded wait gave up
};

// Columns [c_beg, c_end) of split `sp`, in whole chunks.
__device__ __forceinline__ void split_range(const OutArgs& a, uint32_t sp, uint32_t& c_beg, uint32_t& c_end) {
  const uint32_t chunks = a.cp / TN, per = (chunks + a.splits - 1) / a.splits;
  c_beg = min(chunks, sp * per);
  c_end = min(chunks, c_beg + per);
}

// Logits of one chunk: D[128 x 128] = A[128 x 64] . B[128 x 64]^T, issued by one thread.
__device__ __forceinline__ void mma_logits(uint32_t d, const uint8_t* a_tile, const uint8_t* b_tile) {
#pragma unroll
  for (int kk = 0; kk < HK / 16; ++kk)
    mma(d, sdesc(su32(a_tile) + kk * 256u, HK * 16u), sdesc(su32(b_tile) + kk * 256u, HK * 16u), idesc(TM, TN),
        kk > 0 ? 1u : 0u);
}

// The chunk's biases into shared memory (asynchronously; zero past C).
__device__ __forceinline__ void load_bias(float* dst, const float* b3, uint32_t c, uint32_t C) {
  for (uint32_t j = threadIdx.x; j < (uint32_t)TN; j += blockDim.x) {
    const uint32_t col = c * TN + j;
    if (col < C) cp4(dst + j, b3 + col);
    else dst[j] = 0.0f;
  }
}

// 32 logits of this thread's row, bias added; columns past C and invalid
// rows read -inf.
__device__ __forceinline__ void logits32(uint32_t taddr, const float* bias, uint32_t col0, uint32_t C, bool valid_row,
                                         float* v) {
  tmem_ld32(taddr, v);
  if (valid_row && col0 + 32 <= C) {
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] += bias[j];
  } else {
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = (valid_row && col0 + j < C) ? v[j] + bias[j] : -INFINITY;
  }
}

__device__ __forceinline__ float max32(const float* v) {
  float t[16];
#pragma unroll
  for (int j = 0; j < 16; ++j) t[j] = fmaxf(v[j], v[j + 16]);
#pragma unroll
  for (int w = 8; w > 0; w >>= 1)
#pragma unroll
    for (int j = 0; j < w; ++j) t[j] = fmaxf(t[j], t[j + w]);
  return t[0];
}

// Pass 1: per row, the running maximum and exp-sum over the split's columns
// and the target's logit (TOPK = false); or the four largest logits (TOPK).
// Each thread covers one row and one column half of every chunk, so a row's
// results are written as two partial results (index 2 * split + half).
template <bool TOPK>
__global__ void __launch_bounds__(kThreads, 2) out_stats_kernel(OutArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* a_tile = smem;                                        // 128 x 64 bf16: 16 KiB
  uint8_t* b_tile0 = smem + 16384;                               // 128 x 64 bf16: 16 KiB, two buffers
  float* bias = reinterpret_cast<float*>(smem + 16384 + 32768);  // 2 x 128
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, quad = warp & 3, half = warp >> 2;
  const uint32_t row0 = blockIdx.x * TM;
  uint32_t c_beg, c_end;
  split_range(a, blockIdx.y, c_beg, c_end);
  if (tid == 0) {
    bar_init(&bars[0]);
    bar_init(&bars[1]);
  }
  const uint32_t tmem = tmem_alloc(&tmem_slot, warp);
  const uint32_t lanes = tmem + ((uint32_t)(quad * 32) << 16);
  const uint32_t row = row0 + (uint32_t)(quad * 32) + (uint32_t)(tid & 31);
  const bool valid_row = row < a.n;
  const uint32_t tgt = valid_row ? a.s[row].target : 0xFFFFFFFFu;
  float m = -INFINITY, ssum = 0.0f, zt = -INFINITY;
  float tv[4] = {-INFINITY, -INFINITY, -INFINITY, -INFINITY};
  uint32_t ti[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
  uint32_t phases = 0;  // bit b: the parity of buffer b's next phase
  bool ok = true;
  auto load_chunk = [&](uint32_t c, int buf) {
    load_tile(b_tile0 + buf * 16384, a.w3t, HK, c * TN, TN, a.cp, 0, HK);
    load_bias(bias + buf * TN, a.b3, c, a.C);
  };
  if (c_beg < c_end) {
    load_tile(a_tile, a.h2, HK, row0, TM, a.n, 0, HK);
    load_chunk(c_beg, 0);
    cp_commit();
    cp_wait_all();
    fence_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc_after_sync();
      mma_logits(tmem, a_tile, b_tile0);
      commit(&bars[0]);
    }
  }
  for (uint32_t c = c_beg; c < c_end; ++c) {
    const int buf = (int)((c - c_beg) & 1u);
    // the next chunk's operand into the other buffer (its last reader, the
    // MMA of chunk c - 1, finished before that chunk's epilogue)
    if (c + 1 < c_end) {
      load_chunk(c + 1, buf ^ 1);
      cp_commit();
    }
    if (!bar_wait(&bars[buf], (phases >> buf) & 1u)) ok = false;
    phases ^= 1u << buf;
    tc_after_sync();
    if (c + 1 < c_end) {
      cp_wait_all();
      fence_async_smem();
    }
    tc_before_sync();
    __syncthreads();  // the next operand is in place, every thread saw chunk c's MMA complete
    if (c + 1 < c_end && tid == 0) {
      tc_after_sync();
      mma_logits(tmem + (uint32_t)((buf ^ 1) * TN), a_tile, b_tile0 + (buf ^ 1) * 16384);
      commit(&bars[buf ^ 1]);
    }
    // epilogue of chunk c, overlapping the next chunk's MMA
#pragma unroll 1
    for (int sl = 0; sl < 2; ++sl) {
      const uint32_t cl0 = (uint32_t)(half * 64 + sl * 32);  // column within the chunk
      const uint32_t col0 = c * TN + cl0;
      float v[32];
      logits32(lanes + (uint32_t)(buf * TN) + cl0, bias + buf * TN + cl0, col0, a.C, valid_row, v);
      if (TOPK) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const float x = v[j];
          const uint32_t ix = col0 + j;
          if (x > tv[3]) {  // columns arrive in ascending order: ties keep the lower index
            if (x > tv[2]) {
              tv[3] = tv[2], ti[3] = ti[2];
              if (x > tv[1]) {
                tv[2] = tv[1], ti[2] = ti[1];
                if (x > tv[0]) {
                  tv[1] = tv[0], ti[1] = ti[0];
                  tv[0] = x, ti[0] = ix;
                } else {
                  tv[1] = x, ti[1] = ix;
                }
              } else {
                tv[2] = x, ti[2] = ix;
              }
            } else {
              tv[3] = x, ti[3] = ix;
            }
          }
        }
      } else {
        if (tgt - col0 < 32u) {
#pragma unroll
          for (int j = 0; j < 32; ++j)
            if (col0 + j == tgt) zt = v[j];
        }
        const float mx = max32(v);
        if (mx > -INFINITY) {
          const float mn = fmaxf(m, mx), sh = mn * kLog2e;
          float acc0 = ssum * ex2(fmaf(m, kLog2e, -sh)), acc1 = 0.0f;
#pragma unroll
          for (int j = 0; j < 32; j += 2) {
            acc0 += ex2(fmaf(v[j], kLog2e, -sh));
            acc1 += ex2(fmaf(v[j + 1], kLog2e, -sh));
          }
          ssum = acc0 + acc1;
          m = mn;
        }
      }
    }
    tc_before_sync();
    __syncthreads();  // chunk c's TMEM columns are free for chunk c + 2
  }
  if (!ok) atomicOr(a.status, 1u);
  cp_wait_all();  // no copy may still be landing when the CTA exits
  const uint32_t splits2 = a.splits * 2, sp = blockIdx.y * 2 + (uint32_t)half;
  if (valid_row) {
    if (TOPK) {
      float* p = a.part + ((uint64_t)sp * a.n + row) * 8;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        p[2 * k] = tv[k];
        p[2 * k + 1] = __uint_as_float(ti[k]);
      }
    } else {
      a.part[((uint64_t)0 * splits2 + sp) * a.n + row] = m;
      a.part[((uint64_t)1 * splits2 + sp) * a.n + row] = ssum;
      a.part[((uint64_t)2 * splits2 + sp) * a.n + row] = zt;
    }
  }
  tmem_free(tmem, warp);
}

// Pass 1 combined over the partial results: lse per row and the mean loss.
__global__ void out_lse_kernel(const float* __restrict__ part, uint32_t splits, uint32_t n, const rt_mlp_sample* s,
                               uint32_t C, float* __restrict__ lse, float* __restrict__ loss) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  float m = -INFINITY, zt = -INFINITY;
  for (uint32_t k = 0; k < splits; ++k) {
    m = fmaxf(m, part[(uint64_t)k * n + b]);
    zt = fmaxf(zt, part[((uint64_t)2 * splits + k) * n + b]);
  }
  float sum = 0.0f;
  for (uint32_t k = 0; k < splits; ++k) {
    const float mk = part[(uint64_t)k * n + b];
    if (mk > -INFINITY) sum += part[((uint64_t)splits + k) * n + b] * __expf(mk - m);
  }
  const float l = m + logf(sum);
  lse[b] = l;
  if (s[b].target < C) atomicAdd(loss, (l - zt) / (float)n);
}

// Pass 1 (TOPK) combined: the four largest over the partial results' candidates.
__global__ void out_top4_kernel(const float* __restrict__ part, uint32_t splits, uint32_t n, uint32_t* __restrict__ out) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n) return;
  float tv[4] = {-INFINITY, -INFINITY, -INFINITY, -INFINITY};
  uint32_t ti[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
  for (uint32_t k = 0; k < splits; ++k)
    for (int q = 0; q < 4; ++q) {
      const float* p = part + ((uint64_t)k * n + b) * 8 + 2 * q;
      const float x = p[0];
      const uint32_t ix = __float_as_uint(p[1]);
      if (ix == 0xFFFFFFFFu) continue;
      // insert, ties to the lower index
      int pos = 4;
      while (pos > 0 && (x > tv[pos - 1] || (x == tv[pos - 1] && ix < ti[pos - 1]))) --pos;
      if (pos < 4) {
        for (int t = 3; t > pos; --t) tv[t] = tv[t - 1], ti[t] = ti[t - 1];
        tv[pos] = x, ti[pos] = ix;
      }
    }
  for (int q = 0; q < 4; ++q) out[(uint64_t)b * 4 + q] = ti[q];
}

// dz of element (row, col) from its logit z (bias included, -inf where not
// live): (softmax - onehot) / n, with sh = lse * log2(e).
__device__ __forceinline__ float dz_of(float z, float sh, uint32_t col, uint32_t tgt, float inv_n) {
  return (ex2(fmaf(z, kLog2e, -sh)) - (col == tgt ? 1.0f : 0.0f)) * inv_n;
}

// Pass 2: dh2[tile] += dz[tile, split's columns] . W3^T.
__global__ void __launch_bounds__(kThreads, 2) out_dh2_kernel(OutArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* a_tile = smem;                     // h2 tile 128 x 64: 16 KiB
  uint8_t* bz = smem + 16384;                 // W3^T chunk 128 x 64: 16 KiB
  uint8_t* dz = smem + 32768;                 // dz tile 128 x 128 (K-major, K = 128): 32 KiB
  uint8_t* bw = smem + 65536;                 // W3 tile 64 x 128 (K-major, K = 128): 16 KiB
  float* bias = reinterpret_cast<float*>(smem + 81920);
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, quad = warp & 3, half = warp >> 2;
  const uint32_t row0 = blockIdx.x * TM;
  uint32_t c_beg, c_end;
  split_range(a, blockIdx.y, c_beg, c_end);
  if (tid == 0) bar_init(&bar);
  const uint32_t tmem = tmem_alloc(&tmem_slot, warp);
  const uint32_t lanes = tmem + ((uint32_t)(quad * 32) << 16);
  const uint32_t d_h = tmem + TN;  // dh2 accumulator: 64 columns after the logits
  const uint32_t r = (uint32_t)(quad * 32) + (uint32_t)(tid & 31), row = row0 + r;
  const bool valid_row = row < a.n;
  const uint32_t tgt = valid_row ? a.s[row].target : 0xFFFFFFFFu;
  const float sh = valid_row ? a.lse[row] * kLog2e : 0.0f;
  const float inv_n = 1.0f / (float)a.n;
  uint32_t phase = 0;
  bool ok = true;
  load_tile(a_tile, a.h2, HK, row0, TM, a.n, 0, HK);
  for (uint32_t c = c_beg; c < c_end; ++c) {
    load_tile(bz, a.w3t, HK, c * TN, TN, a.cp, 0, HK);
    load_tile(bw, a.w3p, a.cp, 0, HK, HK, c * TN, TN);
    load_bias(bias, a.b3, c, a.C);
    cp_commit();
    cp_wait_all();
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc_after_sync();
      mma_logits(tmem, a_tile, bz);
      commit(&bar);
    }
    if (!bar_wait(&bar, phase)) ok = false;
    phase ^= 1u;
    tc_after_sync();
#pragma unroll 1
    for (int sl = 0; sl < 2; ++sl) {
      const uint32_t cl0 = (uint32_t)(half * 64 + sl * 32);
      const uint32_t col0 = c * TN + cl0;
      float v[32];
      logits32(lanes + cl0, bias + cl0, col0, a.C, valid_row, v);
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        uint32_t w[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int j = q * 8 + 2 * e;
          const float d0 = dz_of(v[j], sh, col0 + j, tgt, inv_n);  // ex2(-inf) = 0: dead columns give 0
          const float d1 = dz_of(v[j + 1], sh, col0 + j + 1, tgt, inv_n);
          const __nv_bfloat162 pr = __floats2bfloat162_rn(d0, d1);
          w[e] = *reinterpret_cast<const uint32_t*>(&pr);
        }
        *reinterpret_cast<uint4*>(dz + koff(r, cl0 + (uint32_t)(q * 8), TN)) = make_uint4(w[0], w[1], w[2], w[3]);
      }
    }
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc_after_sync();
#pragma unroll
      for (int kk = 0; kk < TN / 16; ++kk)
        mma(d_h, sdesc(su32(dz) + kk * 256u, TN * 16u), sdesc(su32(bw) + kk * 256u, TN * 16u), idesc(TM, HK),
            (c > c_beg || kk > 0) ? 1u : 0u);
      commit(&bar);
    }
    if (!bar_wait(&bar, phase)) ok = false;  // dz and bw are read before they are rewritten
    phase ^= 1u;
    tc_after_sync();
  }
  if (!ok) atomicOr(a.status, 1u);
  cp_wait_all();  // no copy may still be landing when the CTA exits
  if (c_beg < c_end) {
    // tcgen05.ld is warp-collective: every lane loads, valid rows store; the
    // two column halves of the CTA take 32 of the 64 columns each
    float v[32];
    tmem_ld32(d_h + ((uint32_t)(quad * 32) << 16) + (uint32_t)(half * 32), v);
    if (valid_row) {
#pragma unroll
      for (int j = 0; j < 32; ++j) atomicAdd(a.dh2 + (uint64_t)row * HK + half * 32 + j, v[j]);
    }
  }
  tmem_free(tmem, warp);
}

// dz^T tile of pass 3 (128 treelet columns x 128 batch rows, K-major along
// the rows) with its K-adjacent core matrices 144 bytes apart instead of
// 128: a warp writes one column's 32 rows, and with 128-byte spacing rows r
// and r + 8 fell on the same banks (40M conflicts of 65M shared-memory
// wavefronts in pass 3); 144 bytes spreads the four groups of 8 rows over
// 16 banks.
constexpr uint32_t kDztLbo = 144, kDztSbo = 16 * kDztLbo;  // 16 K groups per 8-column group
constexpr uint32_t kDztBytes = 16 * kDztSbo;               // 36 KiB
__device__ __forceinline__ uint32_t dzt_off(uint32_t col, uint32_t row) {
  return (col >> 3) * kDztSbo + (row >> 3) * kDztLbo + (col & 7u) * 16u + (row & 7u) * 2u;
}
__device__ __forceinline__ uint64_t sdesc_lbo(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}

// Pass 3: per 128-column chunk and half of the row tiles (blockIdx.y),
// [dW3 | db3]^T += sum over those row tiles of dz^T . [h2 | 1], added into
// the zeroed gradient.
__global__ void __launch_bounds__(kThreads, 2) out_dw3_kernel(OutArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* bz = smem;                          // W3^T chunk 128 x 64: 16 KiB (the CTA's, fixed)
  uint8_t* a_tile = smem + 16384;              // h2 tile 128 x 64: 16 KiB
  uint8_t* dzt = smem + 32768;                 // dz^T 128 x 128 (K-major, K = 128 rows, padded): 36 KiB
  uint8_t* bx = smem + 32768 + kDztBytes;      // [h2 | 1]^T tile 80 x 128 (K-major): 20 KiB
  float* bias = reinterpret_cast<float*>(smem + 32768 + kDztBytes + 20480);
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, quad = warp & 3, half = warp >> 2;
  const uint32_t c = blockIdx.x;  // chunk
  if (tid == 0) bar_init(&bar);
  const uint32_t tmem = tmem_alloc(&tmem_slot, warp);
  const uint32_t lanes = tmem + ((uint32_t)(quad * 32) << 16);
  const uint32_t d_w = tmem + TN;  // [dW3 | db3]^T accumulator: 80 columns after the logits
  const float inv_n = 1.0f / (float)a.n;
  const uint32_t tiles = (a.n + TM - 1) / TM, per = (tiles + gridDim.y - 1) / gridDim.y;
  const uint32_t t_beg = min(tiles, blockIdx.y * per), t_end = min(tiles, t_beg + per);
  const uint32_t r = (uint32_t)(quad * 32) + (uint32_t)(tid & 31);
  uint32_t phase = 0;
  bool ok = true;
  load_tile(bz, a.w3t, HK, c * TN, TN, a.cp, 0, HK);
  load_bias(bias, a.b3, c, a.C);
  for (uint32_t t = t_beg; t < t_end; ++t) {
    const uint32_t row0 = t * TM, row = row0 + r;
    const bool valid_row = row < a.n;
    const uint32_t tgt = valid_row ? a.s[row].target : 0xFFFFFFFFu;
    const float sh = valid_row ? a.lse[row] * kLog2e : 0.0f;
    load_tile(a_tile, a.h2, HK, row0, TM, a.n, 0, HK);
    load_tile(bx, a.h2x, a.ldx, 0, HX, HX, row0, TM);
    cp_commit();
    cp_wait_all();
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc_after_sync();
      mma_logits(tmem, a_tile, bz);
      commit(&bar);
    }
    if (!bar_wait(&bar, phase)) ok = false;
    phase ^= 1u;
    tc_after_sync();
#pragma unroll 1
    for (int sl = 0; sl < 2; ++sl) {
      const uint32_t cl0 = (uint32_t)(half * 64 + sl * 32);
      const uint32_t col0 = c * TN + cl0;
      float v[32];
      logits32(lanes + cl0, bias + cl0, col0, a.C, valid_row, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        // dz^T: element (column cl0 + j, row r)
        *reinterpret_cast<bf16*>(dzt + dzt_off(cl0 + (uint32_t)j, r)) =
            __float2bfloat16_rn(dz_of(v[j], sh, col0 + j, tgt, inv_n));
      }
    }
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc_after_sync();
#pragma unroll
      for (int kk = 0; kk < TM / 16; ++kk)
        mma(d_w, sdesc_lbo(su32(dzt) + kk * 2u * kDztLbo, kDztLbo, kDztSbo), sdesc(su32(bx) + kk * 256u, TM * 16u),
            idesc(TM, HX), (t > t_beg || kk > 0) ? 1u : 0u);
      commit(&bar);
    }
    if (!bar_wait(&bar, phase)) ok = false;
    phase ^= 1u;
    tc_after_sync();
  }
  if (!ok) atomicOr(a.status, 1u);
  cp_wait_all();
  // lane r of the accumulator is column c * 128 + r: 64 weight gradients,
  // then the bias gradient; column half 0 takes k 0..31, half 1 k 32..95
  // (the last load reads past the 80 columns, within the allocation)
  if (t_beg < t_end) {
    const uint32_t col = c * TN + r;
    float v[32];
    for (int q = half; q < (half ? 3 : 1); ++q) {
      tmem_ld32(d_w + ((uint32_t)(quad * 32) << 16) + (uint32_t)(q * 32), v);
      if (col < a.C) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int k = q * 32 + j;
          if (k < HK) atomicAdd(a.dw3 + (uint64_t)k * a.C + col, v[j]);
          else if (k == HK) atomicAdd(a.db3 + col, v[j]);
        }
      }
    }
  }
  tmem_free(tmem, warp);
}

// [h2^T ; ones ; zeros] as BF16 (80 x ldx); columns past n are zero.
__global__ void h2x_kernel(const bf16* __restrict__ h2, uint32_t n, uint32_t ldx, bf16* __restrict__ out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= HX * ldx) return;
  const uint32_t k = i / ldx, b = i % ldx;
  float v = 0.0f;
  if (b < n) v = k < (uint32_t)HK ? __bfloat162float(h2[(uint64_t)b * HK + k]) : (k == (uint32_t)HK ? 1.0f : 0.0f);
  out[i] = __float2bfloat16_rn(v);
}

// W3 (FP32 master, [64][C]) as the two padded BF16 operands: W3 itself
// ([64][cp]) and W3^T ([cp][64]).  One block per 32 columns: W3's rows are
// read and written along the columns, W3^T's through a shared-memory
// transpose (one thread per column wrote 2-byte entries 128 bytes apart).
__global__ void __launch_bounds__(256) w3_operands_kernel(const float* __restrict__ w3, uint32_t C, uint32_t cp,
                                                          bf16* __restrict__ w3t, bf16* __restrict__ w3p) {
  __shared__ __align__(4) bf16 t[32][HK + 2];  // [column][k]: rows 132 bytes apart, no bank conflicts
  const uint32_t c0 = blockIdx.x * 32, tx = threadIdx.x & 31u, ty = threadIdx.x >> 5;
  const uint32_t c = c0 + tx;
  for (uint32_t k = ty; k < (uint32_t)HK; k += 8) {
    const bf16 v = __float2bfloat16_rn(c < C ? w3[(uint64_t)k * C + c] : 0.0f);
    w3p[(uint64_t)k * cp + c] = v;
    t[tx][k] = v;
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < 32u * (HK / 2); i += blockDim.x) {
    const uint32_t cl = i / (HK / 2), kp = i % (HK / 2);
    reinterpret_cast<uint32_t*>(w3t + (uint64_t)(c0 + cl) * HK)[kp] = *reinterpret_cast<const uint32_t*>(&t[cl][2 * kp]);
  }
}

}  // namespace tcm
