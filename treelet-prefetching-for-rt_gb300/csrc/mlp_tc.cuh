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
//   out_dw3_kernel    per 256-column chunk: over every row tile, dz^T, then
//                     [dW3 | db3]^T += dz^T . [h2 | 1] on the tensor cores.
//
// Operands live in shared memory in the canonical K-major layout without
// swizzle: 8-row x 16-byte core matrices, core matrices of one row group
// 128 bytes apart along K (the leading-dimension offset), row groups
// 16 * (K extent) bytes apart (the stride-dimension offset).  One thread issues
// the MMAs and commits them to an mbarrier; every wait is bounded and a wait
// that gives up sets the status word instead of hanging.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace tcm {

using bf16 = __nv_bfloat16;

constexpr int TM = 128;          // rows of a tile (TMEM lanes)
constexpr int TN = 256;          // columns (treelets) of a chunk
constexpr int HK = 64;           // hidden width (K of the logits product)
constexpr int HX = 80;           // [h2 | 1 | 0 ...] rows of the dW3 operand
constexpr uint32_t kTries = 1u << 22;

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

// 512 TMEM columns for the CTA (one warp allocates); returns the base address.
// The .sync.aligned tcgen05 instructions need their whole warp converged,
// hence the __syncwarp before each.
__device__ __forceinline__ uint32_t tmem_alloc(uint32_t* slot, int warp) {
  __syncwarp();
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(su32(slot)));
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
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(base));
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

// Logits of one chunk: D[128 x 256] = A[128 x 64] . B[256 x 64]^T, issued by one thread.
__device__ __forceinline__ void mma_logits(uint32_t d, const uint8_t* a_tile, const uint8_t* b_tile) {
#pragma unroll
  for (int kk = 0; kk < HK / 16; ++kk)
    mma(d, sdesc(su32(a_tile) + kk * 256u, HK * 16u), sdesc(su32(b_tile) + kk * 256u, HK * 16u), idesc(TM, TN),
        kk > 0 ? 1u : 0u);
}

// Pass 1: per row, the running maximum and exp-sum over the split's columns
// and the target's logit (TOPK = false); or the four largest logits (TOPK).
template <bool TOPK>
__global__ void __launch_bounds__(128) out_stats_kernel(OutArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* a_tile = smem;                  // 128 x 64 bf16: 16 KiB
  uint8_t* b_tile0 = smem + 16384;         // 256 x 64 bf16: 32 KiB, two buffers
  float* bias = reinterpret_cast<float*>(smem + 16384 + 65536);  // 2 x 256
  __shared__ __align__(8) uint64_t bars[2];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t row0 = blockIdx.x * TM;
  uint32_t c_beg, c_end;
  split_range(a, blockIdx.y, c_beg, c_end);
  if (tid == 0) {
    bar_init(&bars[0]);
    bar_init(&bars[1]);
  }
  const uint32_t tmem = tmem_alloc(&tmem_slot, warp);
  const uint32_t row = row0 + tid;
  const bool valid_row = row < a.n;
  const uint32_t tgt = valid_row ? a.s[row].target : 0xFFFFFFFFu;
  float m = -INFINITY, ssum = 0.0f, zt = -INFINITY;
  float tv[4] = {-INFINITY, -INFINITY, -INFINITY, -INFINITY};
  uint32_t ti[4] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
  uint32_t phase[2] = {0, 0};
  bool ok = true;
  auto load_chunk = [&](uint32_t c, int buf) {
    load_tile(b_tile0 + buf * 32768, a.w3t, HK, c * TN, TN, a.cp, 0, HK);
    for (uint32_t j = tid; j < TN; j += blockDim.x) {
      const uint32_t col = c * TN + j;
      bias[buf * TN + j] = col < a.C ? a.b3[col] : 0.0f;
    }
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
    if (!bar_wait(&bars[buf], phase[buf])) ok = false;
    phase[buf] ^= 1u;
    tc_after_sync();
    if (c + 1 < c_end) {
      cp_wait_all();
      fence_async_smem();
    }
    tc_before_sync();
    __syncthreads();  // the next operand is in place, every thread saw chunk c's MMA complete
    if (c + 1 < c_end && tid == 0) {
      tc_after_sync();
      mma_logits(tmem + (uint32_t)((buf ^ 1) * TN), a_tile, b_tile0 + (buf ^ 1) * 32768);
      commit(&bars[buf ^ 1]);
    }
    // epilogue of chunk c, overlapping the next chunk's MMA
#pragma unroll 1
    for (int sl = 0; sl < TN / 32; ++sl) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(buf * TN + sl * 32), v);
      const uint32_t col0 = c * TN + sl * 32;
      float mx = -INFINITY;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const bool live = valid_row && col0 + j < a.C;
        v[j] = live ? v[j] + bias[buf * TN + sl * 32 + j] : -INFINITY;
        mx = fmaxf(mx, v[j]);
        if (!TOPK && col0 + j == tgt) zt = v[j];
      }
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
      } else if (mx > -INFINITY) {
        const float mn = fmaxf(m, mx);
        float acc = ssum * __expf(m - mn);
#pragma unroll
        for (int j = 0; j < 32; ++j) acc += __expf(v[j] - mn);
        ssum = acc;
        m = mn;
      }
    }
    tc_before_sync();
    __syncthreads();  // chunk c's TMEM columns are free for chunk c + 2
  }
  if (!ok) atomicOr(a.status, 1u);
  cp_wait_all();  // no copy may still be landing when the CTA exits
  if (valid_row) {
    if (TOPK) {
      float* p = a.part + ((uint64_t)blockIdx.y * a.n + row) * 8;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        p[2 * k] = tv[k];
        p[2 * k + 1] = __uint_as_float(ti[k]);
      }
    } else {
      a.part[((uint64_t)0 * a.splits + blockIdx.y) * a.n + row] = m;
      a.part[((uint64_t)1 * a.splits + blockIdx.y) * a.n + row] = ssum;
      a.part[((uint64_t)2 * a.splits + blockIdx.y) * a.n + row] = zt;
    }
  }
  tmem_free(tmem, warp);
}

// Pass 1 combined over the splits: lse per row and the mean loss.
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

// Pass 1 (TOPK) combined: the four largest over the splits' candidates.
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

// dz of element (row, col) from its logit z (bias included).
__device__ __forceinline__ float dz_of(float z, float lse, uint32_t col, uint32_t tgt, float inv_n, bool live) {
  const float p = __expf(z - lse);
  return live ? (p - (col == tgt ? 1.0f : 0.0f)) * inv_n : 0.0f;
}

// Pass 2: dh2[tile] += dz[tile, split's columns] . W3^T.
__global__ void __launch_bounds__(128) out_dh2_kernel(OutArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* a_tile = smem;                   // h2 tile: 16 KiB
  uint8_t* bz = smem + 16384;               // W3^T chunk: 32 KiB
  uint8_t* dz = smem + 16384 + 32768;       // dz tile 128 x 256 (K-major, K = 256): 64 KiB
  uint8_t* bw = smem + 16384 + 32768 + 65536;  // W3 tile 64 x 256 (K-major): 32 KiB
  float* bias = reinterpret_cast<float*>(smem + 16384 + 32768 + 65536 + 32768);
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t row0 = blockIdx.x * TM;
  uint32_t c_beg, c_end;
  split_range(a, blockIdx.y, c_beg, c_end);
  if (tid == 0) bar_init(&bar);
  const uint32_t tmem = tmem_alloc(&tmem_slot, warp);
  const uint32_t d_h = tmem + TN;  // dh2 accumulator: 64 columns after the logits
  const uint32_t row = row0 + tid;
  const bool valid_row = row < a.n;
  const uint32_t tgt = valid_row ? a.s[row].target : 0xFFFFFFFFu;
  const float l = valid_row ? a.lse[row] : 0.0f;
  const float inv_n = 1.0f / (float)a.n;
  uint32_t phase = 0;
  bool ok = true;
  load_tile(a_tile, a.h2, HK, row0, TM, a.n, 0, HK);
  for (uint32_t c = c_beg; c < c_end; ++c) {
    load_tile(bz, a.w3t, HK, c * TN, TN, a.cp, 0, HK);
    load_tile(bw, a.w3p, a.cp, 0, HK, HK, c * TN, TN);
    for (uint32_t j = tid; j < TN; j += blockDim.x) bias[j] = c * TN + j < a.C ? a.b3[c * TN + j] : 0.0f;
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
    for (int sl = 0; sl < TN / 32; ++sl) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(sl * 32), v);
      const uint32_t col0 = c * TN + sl * 32;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        uint32_t w[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int j = q * 8 + 2 * e;
          const float d0 = dz_of(v[j] + bias[sl * 32 + j], l, col0 + j, tgt, inv_n, valid_row && col0 + j < a.C);
          const float d1 =
              dz_of(v[j + 1] + bias[sl * 32 + j + 1], l, col0 + j + 1, tgt, inv_n, valid_row && col0 + j + 1 < a.C);
          const __nv_bfloat162 pr = __floats2bfloat162_rn(d0, d1);
          w[e] = *reinterpret_cast<const uint32_t*>(&pr);
        }
        *reinterpret_cast<uint4*>(dz + koff((uint32_t)tid, (uint32_t)(sl * 32 + q * 8), TN)) =
            make_uint4(w[0], w[1], w[2], w[3]);
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
    // tcgen05.ld is warp-collective: every lane loads, valid rows store
    float v[32];
    for (int h = 0; h < HK; h += 32) {
      tmem_ld32(d_h + ((uint32_t)(warp * 32) << 16) + (uint32_t)h, v);
      if (valid_row) {
#pragma unroll
        for (int j = 0; j < 32; ++j) atomicAdd(a.dh2 + (uint64_t)row * HK + h + j, v[j]);
      }
    }
  }
  tmem_free(tmem, warp);
}

// Pass 3: per 256-column chunk, [dW3 | db3]^T = sum over row tiles of dz^T . [h2 | 1].
__global__ void __launch_bounds__(128) out_dw3_kernel(OutArgs a) {
  extern __shared__ __align__(1024) uint8_t smem[];
  uint8_t* bz = smem;                         // W3^T chunk: 32 KiB (the CTA's, fixed)
  uint8_t* a_tile = smem + 32768;             // h2 tile: 16 KiB
  uint8_t* dzt = smem + 32768 + 16384;        // dz^T: two 128 x 128 halves (K-major, K = 128): 64 KiB
  uint8_t* bx = smem + 32768 + 16384 + 65536; // [h2 | 1]^T tile 80 x 128 (K-major): 20 KiB
  float* bias = reinterpret_cast<float*>(smem + 32768 + 16384 + 65536 + 20480);
  __shared__ __align__(8) uint64_t bar;
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const uint32_t c = blockIdx.x;  // chunk
  if (tid == 0) bar_init(&bar);
  const uint32_t tmem = tmem_alloc(&tmem_slot, warp);
  const uint32_t d_w0 = tmem + TN, d_w1 = tmem + TN + HX;  // the two halves' accumulators (80 columns each)
  const float inv_n = 1.0f / (float)a.n;
  const uint32_t tiles = (a.n + TM - 1) / TM;
  uint32_t phase = 0;
  bool ok = true;
  load_tile(bz, a.w3t, HK, c * TN, TN, a.cp, 0, HK);
  for (uint32_t j = tid; j < TN; j += blockDim.x) bias[j] = c * TN + j < a.C ? a.b3[c * TN + j] : 0.0f;
  for (uint32_t t = 0; t < tiles; ++t) {
    const uint32_t row0 = t * TM, row = row0 + tid;
    const bool valid_row = row < a.n;
    const uint32_t tgt = valid_row ? a.s[row].target : 0xFFFFFFFFu;
    const float l = valid_row ? a.lse[row] : 0.0f;
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
    for (int sl = 0; sl < TN / 32; ++sl) {
      float v[32];
      tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(sl * 32), v);
      const uint32_t col0 = c * TN + sl * 32;
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const uint32_t cl = (uint32_t)(sl * 32 + j);  // column within the chunk
        const float d = dz_of(v[j] + bias[cl], l, col0 + j, tgt, inv_n, valid_row && col0 + j < a.C);
        // dz^T: element (column cl, row tid) of half cl / 128
        *reinterpret_cast<bf16*>(dzt + (cl >> 7) * 32768u + koff(cl & 127u, (uint32_t)tid, TM)) =
            __float2bfloat16_rn(d);
      }
    }
    fence_async_smem();
    tc_before_sync();
    __syncthreads();
    if (tid == 0) {
      tc_after_sync();
#pragma unroll
      for (int h = 0; h < 2; ++h)
#pragma unroll
        for (int kk = 0; kk < TM / 16; ++kk)
          mma(h ? d_w1 : d_w0, sdesc(su32(dzt) + h * 32768u + kk * 256u, TM * 16u), sdesc(su32(bx) + kk * 256u, TM * 16u),
              idesc(TM, HX), (t > 0 || kk > 0) ? 1u : 0u);
      commit(&bar);
    }
    if (!bar_wait(&bar, phase)) ok = false;
    phase ^= 1u;
    tc_after_sync();
  }
  if (!ok) atomicOr(a.status, 1u);
  // lane tid of each half is column c * 256 + half * 128 + tid: 64 weight
  // gradients, then the bias gradient
  for (int h = 0; h < 2; ++h) {
    const uint32_t col = c * TN + (uint32_t)h * TM + (uint32_t)tid;
    const uint32_t base = (h ? d_w1 : d_w0) + ((uint32_t)(warp * 32) << 16);
    float v[32];
    for (int q = 0; q < 3; ++q) {  // columns 0..95 of the 80: the last load reads past 80, within the allocation
      tmem_ld32(base + (uint32_t)(q * 32), v);
      if (col < a.C) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
          const int k = q * 32 + j;
          if (k < HK) a.dw3[(uint64_t)k * a.C + col] = v[j];
          else if (k == HK) a.db3[col] = v[j];
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

// W3 (FP32 master, [64][C]) as the two padded BF16 operands.
__global__ void w3_operands_kernel(const float* __restrict__ w3, uint32_t C, uint32_t cp, bf16* __restrict__ w3t,
                                   bf16* __restrict__ w3p) {
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (uint64_t)HK * cp) return;
  const uint32_t k = (uint32_t)(i / cp), c = (uint32_t)(i % cp);
  const bf16 v = __float2bfloat16_rn(c < C ? w3[(uint64_t)k * C + c] : 0.0f);
  w3p[i] = v;
  w3t[(uint64_t)c * HK + k] = v;
}

}  // namespace tcm
