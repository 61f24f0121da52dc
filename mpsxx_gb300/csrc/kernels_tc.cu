// Split-precision grouped block GEMM on the 5th-generation tensor cores (sm_103a).
//
// Every FP64 operand element x is split into two TF32 numbers, hi = tf32(x) and
// lo = tf32(x - hi), and a product is formed as hi*hi + hi*lo + lo*hi (the lo*lo
// term is below FP32 resolution): three tcgen05.mma kind::tf32 instructions per
// K=8 step accumulate into one FP32 tile in tensor memory.  The FP32 accumulator
// is flushed into FP64 registers after every (A, B) block pair, so FP32 rounding
// only spans one pair's contraction length; the pair sum, split-K partials and the
// output stay FP64.
//
// CTA: 128 threads, one 128 x 64 output tile (TMEM: 128 lanes x 64 FP32 columns).
// The tile's work is a flat sequence of 32-deep K slices over its (A, B) pairs.
// Pipeline per slice s:
//   * raw FP64 operand tiles arrive in shared memory through cp.async, issued two
//     slices ahead into a double buffer (no register round trip, many bytes in
//     flight per SM);
//   * the threads split the raw tiles into TF32 hi/lo tiles in the K-major
//     no-swizzle core-matrix layout (8 rows x 16 bytes per core matrix);
//   * thread 0 issues 4 x 3 MMAs with shared-memory descriptors and commits them to
//     an mbarrier; the wait on it (bounded by a global-timer deadline) happens just
//     before the next slice overwrites the hi/lo tiles, so loads and the split of
//     slice s+1 overlap the MMAs of slice s.
// The same task/pair plans as the FP64 kernel drive it.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.hpp"

namespace mpsxx {

namespace {

constexpr int BM = kTcTileM;  // 128
constexpr int BN = kTcTileN;  // 64
constexpr int BK = 32;        // TF32 elements per K slice (4 MMA steps of K=8)
constexpr int NTHREADS = 256;  // 8 warps: warp w flushes TMEM lanes 32*(w%4).. and columns 32*(w/4)..
constexpr int CPT = BN / 2;     // accumulator columns per thread
constexpr uint32_t TMEM_COLS = 64;

constexpr int A_TILE_BYTES = BM * BK * 4;  // 16 KB
constexpr int B_TILE_BYTES = BN * BK * 4;  // 8 KB
constexpr int A_RAW_BYTES = BM * BK * 8;   // 32 KB FP64 staging
constexpr int B_RAW_BYTES = BN * BK * 8;   // 16 KB FP64 staging
constexpr int RAW_BYTES = A_RAW_BYTES + B_RAW_BYTES;
constexpr int SMEM_BYTES = 2 * A_TILE_BYTES + 2 * B_TILE_BYTES + 2 * RAW_BYTES + 1024;

// byte offset of element (row, k) in a K-major tile of BK columns made of 8x4 core matrices
__device__ __forceinline__ uint32_t core_off(int row, int k) {
  return (uint32_t)(((row >> 3) * (BK / 4) + (k >> 2)) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint32_t tf32_rna(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

// shared-memory matrix descriptor: start, leading (K-direction) and stride
// (M/N-direction) byte offsets between core matrices, sm_100 version bits, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor: D = F32, A = B = TF32, both K-major, N = BN, M = BM
__host__ __device__ constexpr uint32_t tf32_idesc() {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.u32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// bounded parity wait: false when the deadline passed
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase, uint64_t deadline) {
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(phase)
        : "memory");
    if (done) return true;
    if (global_ns() > deadline) return false;
  }
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void cp_async8(uint32_t dst, const double* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

struct SliceCursor {
  int p;   // pair index
  int k0;  // first K element of the slice inside the pair
};

__device__ __forceinline__ void advance(SliceCursor& c, const DGemmPair* pairs) {
  c.k0 += BK;
  if (c.k0 >= pairs[c.p].k) {
    ++c.p;
    c.k0 = 0;
  }
}

// Stage one slice of raw FP64 operands (zero outside the block) into shared memory:
// A as [BM][BK] and B^T as [BN][BK], row-major.
__device__ __forceinline__ void load_slice(const SliceCursor& c, const DGemmPair* __restrict__ pairs,
                                           const DGemmTask& task, int m0, int n0, int transa, int transb,
                                           const double* __restrict__ A, const double* __restrict__ B,
                                           double* a_raw, double* b_raw) {
  const DGemmPair pr = pairs[c.p];
  const int k0 = c.k0;
  const uint32_t a_s = smem_u32(a_raw), b_s = smem_u32(b_raw);
  if (!transa) {
    for (int e = threadIdx.x; e < BM * BK; e += NTHREADS) {
      const int r = e / BK, kk = e % BK;
      const int gr = m0 + r, gk = k0 + kk;
      if (gr < task.m && gk < pr.k)
        cp_async8(a_s + (uint32_t)(r * BK + kk) * 8, A + pr.a_off + (int64_t)gr * pr.lda + gk);
      else
        a_raw[r * BK + kk] = 0.0;
    }
  } else {
    for (int e = threadIdx.x; e < BM * BK; e += NTHREADS) {
      const int r = e % BM, kk = e / BM;
      const int gr = m0 + r, gk = k0 + kk;
      if (gr < task.m && gk < pr.k)
        cp_async8(a_s + (uint32_t)(r * BK + kk) * 8, A + pr.a_off + (int64_t)gk * pr.lda + gr);
      else
        a_raw[r * BK + kk] = 0.0;
    }
  }
  if (!transb) {
    for (int e = threadIdx.x; e < BN * BK; e += NTHREADS) {
      const int cc = e % BN, kk = e / BN;
      const int gc = n0 + cc, gk = k0 + kk;
      if (gc < task.n && gk < pr.k)
        cp_async8(b_s + (uint32_t)(cc * BK + kk) * 8, B + pr.b_off + (int64_t)gk * pr.ldb + gc);
      else
        b_raw[cc * BK + kk] = 0.0;
    }
  } else {
    for (int e = threadIdx.x; e < BN * BK; e += NTHREADS) {
      const int cc = e / BK, kk = e % BK;
      const int gc = n0 + cc, gk = k0 + kk;
      if (gc < task.n && gk < pr.k)
        cp_async8(b_s + (uint32_t)(cc * BK + kk) * 8, B + pr.b_off + (int64_t)gc * pr.ldb + gk);
      else
        b_raw[cc * BK + kk] = 0.0;
    }
  }
}

__device__ __forceinline__ void split_tile(const double* raw, int rows, uint8_t* hi, uint8_t* lo) {
  for (int e = threadIdx.x; e < rows * BK; e += NTHREADS) {
    const int r = e / BK, kk = e % BK;
    const double v = raw[e];
    const uint32_t h = tf32_rna(static_cast<float>(v));
    const uint32_t l = tf32_rna(static_cast<float>(v - static_cast<double>(__uint_as_float(h))));
    const uint32_t off = core_off(r, kk);
    *reinterpret_cast<uint32_t*>(hi + off) = h;
    *reinterpret_cast<uint32_t*>(lo + off) = l;
  }
}

__global__ void __launch_bounds__(NTHREADS, 1)
    gemm_tc_kernel(int transa, int transb, double alpha, const double* __restrict__ A,
                   const double* __restrict__ B, double* __restrict__ C, const DTile* __restrict__ tiles,
                   const DGemmTask* __restrict__ tasks, const DGemmPair* __restrict__ pairs,
                   double* __restrict__ partial, int* __restrict__ err, uint64_t timeout_ns) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  uint8_t* a_hi = base;
  uint8_t* a_lo = a_hi + A_TILE_BYTES;
  uint8_t* b_hi = a_lo + A_TILE_BYTES;
  uint8_t* b_lo = b_hi + B_TILE_BYTES;
  double* raw0 = reinterpret_cast<double*>(b_lo + B_TILE_BYTES);
  double* raw1 = raw0 + RAW_BYTES / 8;
  __shared__ __align__(8) uint64_t mbar;
  __shared__ uint32_t tmem_slot;

  const DTile t = tiles[blockIdx.x];
  const DGemmTask task = tasks[t.task];
  const int m0 = t.tm * BM, n0 = t.tn * BN;
  const int warp = threadIdx.x >> 5;

  // slices of this tile
  int nslice = 0;
  for (int p = t.p0; p < t.p1; ++p) nslice += (pairs[p].k + BK - 1) / BK;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;
  const uint32_t mb = smem_u32(&mbar);
  const uint32_t idesc = tf32_idesc();
  const uint64_t deadline = global_ns() + timeout_ns;
  const int quarter = warp & 3, half = warp >> 2;
  const uint32_t lane_addr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(half * CPT);

  double acc[CPT];
#pragma unroll
  for (int j = 0; j < CPT; ++j) acc[j] = 0.0;

  // prologue: slices 0 and 1 in flight
  SliceCursor ld{t.p0, 0};
  for (int s = 0; s < 2; ++s) {
    if (s < nslice) {
      double* raw = s ? raw1 : raw0;
      load_slice(ld, pairs, task, m0, n0, transa, transb, A, B, raw, raw + A_RAW_BYTES / 8);
      advance(ld, pairs);
    }
    cp_async_commit();
  }

  uint32_t phase = 0;
  bool ok = true;
  SliceCursor cv{t.p0, 0};
  for (int s = 0; s < nslice; ++s) {
    double* raw = (s & 1) ? raw1 : raw0;
    cp_async_wait1();  // slice s has landed
    if (s > 0) {
      // MMAs of slice s-1 read the hi/lo tiles: they must be complete before the split
      ok = __syncthreads_and(mbar_wait(mb, phase, deadline) ? 1 : 0) != 0;
      phase ^= 1u;
      if (!ok) break;
      if (cv.k0 == 0) {
        // slice s starts a new pair: the accumulator holds the previous pair; flush it to FP64
        asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
        for (int c0 = 0; c0 < CPT; c0 += 16) {
          float v[16];
          tmem_ld16(lane_addr + c0, v);
          asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
          for (int i = 0; i < 16; ++i) acc[c0 + i] += static_cast<double>(v[i]);
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
      }
    } else {
      __syncthreads();
    }
    split_tile(raw, BM, a_hi, a_lo);
    split_tile(raw + A_RAW_BYTES / 8, BN, b_hi, b_lo);
    // generic-proxy stores -> visible to the tensor core (async proxy)
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    // the raw buffer is free again: stage slice s+2 into it
    if (s + 2 < nslice) {
      load_slice(ld, pairs, task, m0, n0, transa, transb, A, B, raw, raw + A_RAW_BYTES / 8);
      advance(ld, pairs);
    }
    cp_async_commit();
    if (threadIdx.x == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t lbo = 128, sbo = (BK / 4) * 128;
      const bool first = (cv.k0 == 0);
#pragma unroll
      for (int ks = 0; ks < BK / 8; ++ks) {
        const uint32_t koff = ks * 2 * 128;  // two core matrices per K=8 step
        const uint64_t ah = smem_desc(smem_u32(a_hi) + koff, lbo, sbo);
        const uint64_t al = smem_desc(smem_u32(a_lo) + koff, lbo, sbo);
        const uint64_t bh = smem_desc(smem_u32(b_hi) + koff, lbo, sbo);
        const uint64_t bl = smem_desc(smem_u32(b_lo) + koff, lbo, sbo);
        mma_tf32(tmem, ah, bh, idesc, (first && ks == 0) ? 0u : 1u);
        mma_tf32(tmem, ah, bl, idesc, 1u);
        mma_tf32(tmem, al, bh, idesc, 1u);
      }
      mma_commit(mb);
    }
    advance(cv, pairs);
  }
  cp_async_wait0();
  if (ok && nslice > 0) {
    ok = __syncthreads_and(mbar_wait(mb, phase, deadline) ? 1 : 0) != 0;
    if (ok) {
      asm volatile("tcgen05.fence::after_thread_sync;");
#pragma unroll
      for (int c0 = 0; c0 < CPT; c0 += 16) {
        float v[16];
        tmem_ld16(lane_addr + c0, v);
        asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
        for (int i = 0; i < 16; ++i) acc[c0 + i] += static_cast<double>(v[i]);
      }
    }
  }

  if (!ok) {
    if (threadIdx.x == 0) atomicExch(err, 1);
  } else {
    // this thread owns tile row 32*quarter + lane and columns CPT*half .. CPT*half + CPT-1
    const int row = quarter * 32 + (threadIdx.x & 31);
    const int col0 = half * CPT;
    const int r = m0 + row;
    if (t.slot >= 0) {
      double* part = partial + (int64_t)t.slot * (BM * BN) + (int64_t)row * BN + col0;
#pragma unroll
      for (int j = 0; j < CPT; ++j) part[j] = acc[j];
    } else if (r < task.m) {
      double* dst = C + task.c_off + (int64_t)r * task.ldc + n0 + col0;
#pragma unroll
      for (int j = 0; j < CPT; ++j)
        if (n0 + col0 + j < task.n) dst[j] += alpha * acc[j];
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

__global__ void __launch_bounds__(256) gemm_tc_reduce_kernel(const DReduce* __restrict__ red,
                                                             const DGemmTask* __restrict__ tasks, double alpha,
                                                             const double* __restrict__ partial,
                                                             double* __restrict__ C) {
  const DReduce rd = red[blockIdx.x];
  const DGemmTask task = tasks[rd.task];
  const int m0 = rd.tm * BM, n0 = rd.tn * BN;
  for (int e = threadIdx.x; e < BM * BN; e += blockDim.x) {
    const int r = m0 + e / BN, c = n0 + e % BN;
    if (r >= task.m || c >= task.n) continue;
    double s = 0.0;
    for (int k = 0; k < rd.nslot; ++k) s += partial[(int64_t)(rd.slot0 + k) * (BM * BN) + e];
    C[task.c_off + (int64_t)r * task.ldc + c] += alpha * s;
  }
}

}  // namespace

int tc_smem_bytes() { return SMEM_BYTES; }

void launch_gemm_tc(int transa, int transb, double alpha, const double* A, const double* B, double* C,
                    const DTile* tiles, int ntiles, const DGemmTask* tasks, const DGemmPair* pairs, double* partial,
                    int* err, cudaStream_t st) {
  if (ntiles <= 0) return;
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    configured = true;
  }
  const uint64_t timeout_ns = 2000000000ull;  // 2 s per tile
  gemm_tc_kernel<<<ntiles, NTHREADS, SMEM_BYTES, st>>>(transa, transb, alpha, A, B, C, tiles, tasks, pairs, partial,
                                                       err, timeout_ns);
}

void launch_gemm_tc_reduce(const DReduce* red, int nred, const DGemmTask* tasks, double alpha, const double* partial,
                           double* C, cudaStream_t st) {
  if (nred <= 0) return;
  gemm_tc_reduce_kernel<<<nred, 256, 0, st>>>(red, tasks, alpha, partial, C);
}

}  // namespace mpsxx
