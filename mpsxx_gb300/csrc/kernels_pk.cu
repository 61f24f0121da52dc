// Split-precision grouped block GEMM over pre-packed operands (sm_103a).
//
// Operands are packed once into the tensor-core tile format: a block used as the
// A operand (rows x K) or as B (rows = output columns) becomes ceil(rows/128) x
// ceil(K/32) tiles of 32 KB [hi TF32 128x32 | lo TF32 128x32] (a last tile of at most
// 64 rows is packed compact: 16 KB), each half in the K-major no-swizzle core-matrix
// layout the MMA descriptors address (8 rows x 16 bytes per core matrix).
// hi = tf32(x), lo = tf32(x - hi); a product is hi*hi + hi*lo + lo*hi.
//
// An intermediate that one GEMM writes and the next reads once (stage 1 -> stage 2 of
// H_eff * psi) is written either in that packed hi|lo format or as FP32 values (16 KB
// A tiles, half the bytes) that the next GEMM splits on chip — hi and lo from an FP32
// value carry no more than the value itself; the split costs shared-memory traffic, so
// the plan's autotuner picks the format.
//
// GEMM CTA (384 threads, warp-specialised), one output tile of 128 x 128:
//   warp 0 lane 0 : producer — per K slice, one bulk copy (TMA engine) of the A tile
//                   and one of the B tile into a 3-stage shared-memory ring,
//                   completion counted in bytes on the stage's "full" mbarrier;
//   warps 2-3     : (FP32 A tiles only) converter — split the landed A tile in place
//                   into hi | lo, fence it for the tensor core (async proxy) and mark
//                   the stage "converted";
//   warp 1 lane 0 : MMA issuer — per K-step of 8, A_hi x [B_hi; B_lo] (N = 256) and
//                   A_lo x B_hi (N = 128), tcgen05.mma kind::tf32 (M = 64 / N halved
//                   on tail tiles), into one of two TMEM accumulators (alternating per
//                   group of block pairs); commits release the stage ("empty") and, at
//                   the end of a group, hand the accumulator to the epilogue ("acc_full");
//   warps 4-11    : epilogue — warp 4 + 4 c + q reads TMEM lane quarter q, output
//                   columns [64 c, 64 c + 64): per group, tcgen05.ld of the FP32
//                   accumulator into FP64 registers, then release it ("acc_empty"); at
//                   the end write FP64 C (+=), an FP64 split-K partial, or the packed A
//                   tiles of the next GEMM (stage-1 output).
// Every wait is bounded by a global-timer deadline; a timeout sets a shared abort
// flag that ends all roles and the device error flag the host checks.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.hpp"

namespace mpsxx {

namespace {

constexpr int BM = kTcTileM;  // 128
constexpr int BN = kTcTileN;  // 128
constexpr int BK = kPkTileK;  // 32
constexpr int NTHREADS = 384;
constexpr int EPI_THREADS = 256;  // warps 4-11
constexpr int STAGES = 3;
constexpr uint32_t A_BYTES = kPkTileABytes;  // 32 KB
constexpr uint32_t A1_BYTES = kPkTileA1Bytes;  // 16 KB (FP32 A tile)
constexpr int CONV_THREADS = 64;               // warps 2-3
constexpr uint32_t B_BYTES = kPkTileBBytes;  // 32 KB
constexpr uint32_t B1_BYTES = kPkTileB1Bytes;  // 16 KB (FP32 B tile)
constexpr uint32_t STAGE_BYTES = A_BYTES + B_BYTES;
constexpr int SMEM_BYTES = STAGES * STAGE_BYTES + 1024;
// Each K step is two MMAs: A_hi x [B_hi; B_lo] as one N = 2 Nt operand (the packed B
// tile is exactly that: hi rows then lo rows; Nt = 128, or 64 on a tail tile) into
// accumulator columns [0, 2 Nt), and A_lo x B_hi (N = Nt) into columns [0, Nt).  The
// product is then columns [0, Nt) + [Nt, 2 Nt).  Fewer, wider MMAs read fewer operand
// bytes from shared memory, whose bandwidth (with the bulk copies and the on-chip
// split) bounds the kernel.
constexpr uint32_t ACC_COLS = 2 * BN;             // one accumulator: 256 columns
constexpr uint32_t TMEM_COLS = 2 * ACC_COLS;       // two accumulators: all 512 columns
// Consecutive block pairs of a tile accumulate in the FP32 tensor-memory tile until
// their summed contraction length reaches FLUSH_K; then the group is flushed into
// the FP64 accumulators.  This bounds the FP32 accumulation length (rounding ~
// sqrt(FLUSH_K) * 2^-24, below the TF32 split error) while keeping FP64 work —
// GB300's narrowest pipe — off the per-pair path.
constexpr int FLUSH_K = kFlushK;

// group boundary: after pair p (with running contraction length kacc) of a tile
__device__ __forceinline__ bool group_ends(int kacc, int p, int p_last) { return kacc >= FLUSH_K || p == p_last; }

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

__device__ __forceinline__ void split2(double v, uint32_t& h, uint32_t& l) {
  h = tf32_rna(static_cast<float>(v));
  l = tf32_rna(static_cast<float>(v - static_cast<double>(__uint_as_float(h))));
}

__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

__host__ __device__ constexpr uint32_t tf32_idesc(int m, int n) {
  return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
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

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(done)
      : "r"(mbar), "r"(parity)
      : "memory");
  return done != 0;
}

// bounded wait; false on timeout (the deadline is checked on entry too, so a limit
// already past always ends the kernel) or when another role aborted
__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, uint64_t deadline,
                                          volatile int* abort_flag) {
  if (global_ns() > deadline) {
    *abort_flag = 1;
    return false;
  }
  while (!mbar_try(mbar, parity)) {
    if (*abort_flag) return false;
    if (global_ns() > deadline) {
      *abort_flag = 1;
      return false;
    }
  }
  return true;
}

// bounded wait that ignores the abort flag: draining the kernel's own asynchronous
// work (bulk copies, MMAs) before it frees tensor memory and exits
__device__ __forceinline__ void mbar_drain(uint32_t mbar, uint32_t parity, uint64_t deadline) {
  while (!mbar_try(mbar, parity) && global_ns() <= deadline) {
  }
}
constexpr uint64_t DRAIN_NS = 1000000000ull;  // 1 s

__device__ __forceinline__ void mbar_init(uint32_t mbar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(mbar), "r"(count));
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(mbar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
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

__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float* v) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

// FP32 values at base (n16 x 16 bytes) -> hi = tf32(x) in place, lo = tf32(x - hi) at
// base + lo_off; the converter's CONV_THREADS threads share the work.
__device__ __forceinline__ void split_in_place(uint8_t* base, uint32_t lo_off, int n16, int ct) {
  uint4* hi = reinterpret_cast<uint4*>(base);
  uint4* lo = reinterpret_cast<uint4*>(base + lo_off);
#pragma unroll 4
  for (int i = ct; i < n16; i += CONV_THREADS) {
    const uint4 x = hi[i];
    uint4 h, l;
    h.x = tf32_rna(__uint_as_float(x.x));
    h.y = tf32_rna(__uint_as_float(x.y));
    h.z = tf32_rna(__uint_as_float(x.z));
    h.w = tf32_rna(__uint_as_float(x.w));
    l.x = tf32_rna(__uint_as_float(x.x) - __uint_as_float(h.x));
    l.y = tf32_rna(__uint_as_float(x.y) - __uint_as_float(h.y));
    l.z = tf32_rna(__uint_as_float(x.z) - __uint_as_float(h.z));
    l.w = tf32_rna(__uint_as_float(x.w) - __uint_as_float(h.w));
    hi[i] = h;
    lo[i] = l;
  }
}

__global__ void __launch_bounds__(NTHREADS, 1)
    gemm_pk_kernel(const uint8_t* __restrict__ Apk, const uint8_t* __restrict__ Bpk, double alpha,
                   double* __restrict__ C, uint8_t* __restrict__ Cpk, const DTile* __restrict__ tiles, int ntiles,
                   const DGemmTask* __restrict__ tasks, const DPkPair* __restrict__ pairs,
                   double* __restrict__ partial, int out_packed, int single, int* __restrict__ err,
                   uint64_t timeout_ns, const int64_t* __restrict__ row_map) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  uint8_t* ring = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __shared__ __align__(8) uint64_t full_bar[STAGES];
  __shared__ __align__(8) uint64_t empty_bar[STAGES];
  __shared__ __align__(8) uint64_t conv_bar[STAGES];
  __shared__ __align__(8) uint64_t drain_bar;
  __shared__ __align__(8) uint64_t accf_bar[2];
  __shared__ __align__(8) uint64_t acce_bar[2];
  __shared__ uint32_t tmem_slot;
  __shared__ volatile int abort_flag;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                 "r"(TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (threadIdx.x == 32) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&full_bar[s]), 1);
      mbar_init(smem_u32(&empty_bar[s]), 1);
      mbar_init(smem_u32(&conv_bar[s]), CONV_THREADS);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(smem_u32(&accf_bar[b]), 1);
      mbar_init(smem_u32(&acce_bar[b]), EPI_THREADS);
    }
    mbar_init(smem_u32(&drain_bar), 1);
    abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_slot;
  const uint64_t deadline = global_ns() + timeout_ns;
  const bool a_single = single & kSingleA, b_single = single & kSingleB;
  const int conv = single & (kSingleA | kSingleB);
  const uint32_t a_bytes = a_single ? A1_BYTES : A_BYTES;  // A tile in global memory
  const uint32_t b_bytes = b_single ? B1_BYTES : B_BYTES;  // B tile in global memory

  // Persistent: the CTA walks tiles blockIdx.x, blockIdx.x + gridDim.x, ...; every
  // role walks the same sequence, so slice and pair counters continue across tiles.
  if (warp == 0) {
    // ---------------- producer ----------------
    if (lane == 0) {
      int slice = 0;
      // descriptors are loaded one pair (and one tile) ahead, so that their latency
      // hides behind the current pair's copies
      DTile t_next = blockIdx.x < ntiles ? tiles[blockIdx.x] : DTile{};
      for (int ti = blockIdx.x; ti < ntiles && !abort_flag; ti += gridDim.x) {
        const DTile t = t_next;
        if (ti + (int)gridDim.x < ntiles) t_next = tiles[ti + gridDim.x];
        DPkPair pr_next = t.p0 < t.p1 ? pairs[t.p0] : DPkPair{};
        for (int p = t.p0; p < t.p1 && !abort_flag; ++p) {
          const DPkPair pr = pr_next;
          if (p + 1 < t.p1) pr_next = pairs[p + 1];
          for (int ks = 0; ks < pr.nks; ++ks, ++slice) {
            const int s = slice % STAGES;
            const uint32_t round = slice / STAGES;
            if (!mbar_wait(smem_u32(&empty_bar[s]), (round & 1u) ^ 1u, deadline, &abort_flag)) break;
            const uint32_t fb = smem_u32(&full_bar[s]);
            // a 64-row tail tile is packed compact: half the bytes; its hi and lo
            // halves (split format) land where the MMA expects a 128-row tile's
            const uint32_t at = t.h64 ? a_bytes / 2 : a_bytes;
            // a block's last column tile is compact: [hi nt | lo nt] (or nt FP32 rows)
            const uint32_t bt = b_bytes / BN * t.nt;
            mbar_expect_tx(fb, at + bt);
            const uint32_t dst = smem_u32(ring + s * STAGE_BYTES);
            const uint8_t* asrc = Apk + pr.a_pk + (int64_t)t.tm * pr.nks * a_bytes + (int64_t)ks * at;
            if (t.h64 && !a_single) {
              bulk_g2s(dst, asrc, at / 2, fb);
              bulk_g2s(dst + A_BYTES / 2, asrc + at / 2, at / 2, fb);
            } else {
              bulk_g2s(dst, asrc, at, fb);
            }
            bulk_g2s(dst + A_BYTES, Bpk + pr.b_pk + (int64_t)t.tn * pr.nks * b_bytes + (int64_t)ks * bt, bt, fb);
          }
        }
      }
      // every bulk copy issued lands before the kernel exits (after an abort the
      // consumers no longer wait for them): the last STAGES slices' phases
      const uint64_t dl = global_ns() + DRAIN_NS;
      for (int k = slice - STAGES < 0 ? 0 : slice - STAGES; k < slice; ++k)
        mbar_drain(smem_u32(&full_bar[k % STAGES]), (uint32_t)(k / STAGES) & 1u, dl);
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer ----------------
    if (lane == 0) {

      const uint32_t lbo = 128, sbo = (BK / 4) * 128;
      // Descriptors of the stages' A and B tiles, built once: the start address sits in
      // the low 14 bits (address >> 4), so the K steps and the lo halves are immediate
      // additions (every shared address stays below 2^18: no carry out of the field).
      uint64_t dA[STAGES], dB[STAGES];
#pragma unroll
      for (int s = 0; s < STAGES; ++s) {
        dA[s] = smem_desc(smem_u32(ring + s * STAGE_BYTES), lbo, sbo);
        dB[s] = smem_desc(smem_u32(ring + s * STAGE_BYTES + A_BYTES), lbo, sbo);
      }
      int slice = 0, gc = 0;
      bool ok = true;
      DTile t_next = blockIdx.x < ntiles ? tiles[blockIdx.x] : DTile{};
      for (int ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x) {
        const DTile t = t_next;
        if (ti + (int)gridDim.x < ntiles) t_next = tiles[ti + gridDim.x];
        const int mt = t.h64 ? 64 : BM, nt = t.nt;
        const uint32_t idesc_w = tf32_idesc(mt, 2 * nt), idesc = tf32_idesc(mt, nt);
        int kacc = 0;
        int nks_next = t.p0 < t.p1 ? pairs[t.p0].nks : 0;
        for (int p = t.p0; p < t.p1 && ok; ++p) {
          const int nks = nks_next;
          if (p + 1 < t.p1) nks_next = pairs[p + 1].nks;
          const int b = gc & 1;
          const bool group_start = (kacc == 0);
          if (group_start) {
            // the epilogue must have drained this accumulator (group gc-2)
            if (!mbar_wait(smem_u32(&acce_bar[b]), ((gc >> 1) & 1u) ^ 1u, deadline, &abort_flag)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
          }
          const uint32_t d = tmem + b * ACC_COLS;
          for (int ks = 0; ks < nks; ++ks, ++slice) {
            const int s = slice % STAGES;
            const uint32_t round = slice / STAGES;
            if (!mbar_wait(smem_u32(conv ? &conv_bar[s] : &full_bar[s]), round & 1u, deadline, &abort_flag)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;");
            uint64_t a0d = dA[0], b0d = dB[0];
#pragma unroll
            for (int q = 1; q < STAGES; ++q)
              if (s == q) {
                a0d = dA[q];
                b0d = dB[q];
              }
#pragma unroll
            for (int kk = 0; kk < BK / 8; ++kk) {
              const uint64_t koff = (uint64_t)(kk * 256) >> 4;
              const uint64_t ah = a0d + koff;
              const uint64_t al = a0d + ((A_BYTES / 2) >> 4) + koff;
              const uint64_t bh = b0d + koff;  // [B_hi; B_lo] for the wide MMA, B_hi for the other
              mma_tf32(d, ah, bh, idesc_w, (group_start && ks == 0 && kk == 0) ? 0u : 1u);
              mma_tf32(d, al, bh, idesc, 1u);
            }
            mma_commit(smem_u32(&empty_bar[s]));  // stage free once these MMAs completed
          }
          if (!ok) break;
          kacc += nks * BK;
          if (group_ends(kacc, p, t.p1 - 1)) {
            mma_commit(smem_u32(&accf_bar[b]));  // group accumulated
            ++gc;
            kacc = 0;
          }
        }
      }
      // every MMA issued has completed before tensor memory is freed
      mma_commit(smem_u32(&drain_bar));
      mbar_drain(smem_u32(&drain_bar), 0u, global_ns() + DRAIN_NS);
    }
  } else if (warp == 2 || warp == 3) {
    // ---------------- converter (FP32 A and/or B tiles) ----------------
    if (conv) {
      const int ct = threadIdx.x - 64;
      int slice = 0;
      bool ok = true;
      DTile t_next = blockIdx.x < ntiles ? tiles[blockIdx.x] : DTile{};
      for (int ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x) {
        const DTile t = t_next;
        if (ti + (int)gridDim.x < ntiles) t_next = tiles[ti + gridDim.x];
        int nks_next = t.p0 < t.p1 ? pairs[t.p0].nks : 0;
        for (int p = t.p0; p < t.p1 && ok; ++p) {
          const int nks = nks_next;
          if (p + 1 < t.p1) nks_next = pairs[p + 1].nks;
          for (int ks = 0; ks < nks; ++ks, ++slice) {
            const int s = slice % STAGES;
            const uint32_t round = slice / STAGES;
            if (!mbar_wait(smem_u32(&full_bar[s]), round & 1u, deadline, &abort_flag)) {
              ok = false;
              break;
            }
            // element-wise, so the core-matrix layout carries over: hi in place, lo at
            // the same offset in the operand's lo half.  A: the lo half starts half a
            // 128-row tile in (where the M = 64 MMA reads it too); B: right after the hi
            // rows, which the wide N = 2 Nt MMA reads as one operand ([B_hi; B_lo]).
            if (a_single)
              split_in_place(ring + s * STAGE_BYTES, A_BYTES / 2, static_cast<int>(A1_BYTES / 16) >> (t.h64 ? 1 : 0),
                             ct);
            if (b_single)
              split_in_place(ring + s * STAGE_BYTES + A_BYTES, B1_BYTES / BN * t.nt,
                             static_cast<int>(B1_BYTES / BN * t.nt / 16), ct);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            mbar_arrive(smem_u32(&conv_bar[s]));
          }
        }
      }
    }
  } else if (warp >= 4) {
    // ---------------- epilogue ----------------
    const int q = (warp - 4) & 3;   // TMEM lane quarter (warp id mod 4)
    const int ch = (warp - 4) >> 2;  // column half: output columns [64 ch, 64 ch + 64)
    int gc = 0;
    bool ok = true;
    for (int ti = blockIdx.x; ti < ntiles && ok; ti += gridDim.x) {
      const DTile t = tiles[ti];
      const DGemmTask task = tasks[t.task];
      // the tile row this thread's TMEM lane holds: 128-row tiles, lane 32 q + i holds
      // row 32 q + i; M = 64 tiles, lane 32 q + i holds row 16 q + i for i < 16 (and
      // nothing for i >= 16); -1: no row
      const int row = t.h64 ? (lane < 16 ? q * 16 + lane : -1) : q * 32 + lane;
      const int r = t.tm * BM + row;
      const int nt = t.nt;                // output columns of the tile
      const bool cols = 64 * ch < nt;     // this warp has columns (not on a 64-column tail)
      const uint32_t c1 = 64 * ch, c2 = nt + 64 * ch;  // its columns in both accumulator parts
      if (out_packed) {
        // stage-1 output (one group): FP32 straight from tensor memory, re-split into
        // the packed A tiles of the next GEMM; output columns [128 tn + 64 ch, +64) are
        // its K slices 4 tn + 2 ch and 4 tn + 2 ch + 1, ldc carries that GEMM's slices
        // per row tile
        int kacc = 0;
        for (int p = t.p0; p < t.p1 && ok; ++p) {
          kacc += pairs[p].nks * BK;
          if (!group_ends(kacc, p, t.p1 - 1)) continue;
          kacc = 0;
          const int b = gc & 1;
          if (!mbar_wait(smem_u32(&accf_bar[b]), (gc >> 1) & 1u, deadline, &abort_flag)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + b * ACC_COLS;
          const bool single = out_packed == kOutPackedSingle;
          const uint32_t ot_bytes = single ? A1_BYTES : A_BYTES;  // output tile (128 rows)
          // the next GEMM's A tile grid for this row tile: a 64-row tail tile is
          // compact (half the bytes, its lo half a quarter tile in)
          uint32_t ts = t.h64 ? ot_bytes / 2 : ot_bytes;
          uint8_t* tile0 = Cpk + task.c_off + (int64_t)t.tm * task.ldc * ot_bytes;
          int row_d = row, ldc = task.ldc;  // destination row in its tile, K slices of its block
          if (row_map != nullptr) {
            // stacked panel: this row's output block and row from the row map
            row_d = -1;
            if (row >= 0) {
              const int64_t e = row_map[(int64_t)pairs[t.p0].pad + (int64_t)t.tm * BM + row];
              if (e >= 0) {
                const DGemmTask dt = tasks[static_cast<int>(e >> 32)];
                const int br = static_cast<int>(e & 0xffffffffll), tmd = br / BM;
                row_d = br % BM;
                ts = tail64(dt.m, tmd) ? ot_bytes / 2 : ot_bytes;
                tile0 = Cpk + dt.c_off + (int64_t)tmd * dt.ldc * ot_bytes;
                ldc = dt.ldc;
              }
            }
          }
          const uint32_t lo_off = ts / 2;
          const float fa = static_cast<float>(alpha);
          // 16 columns at a time: half a K slice of the next GEMM
#pragma unroll 1
          for (int hq = 0; hq < 4 && cols; ++hq) {
            const int h = hq >> 1, k0 = (hq & 1) * 16;
            float v[16], w[16];
            tmem_ld16(taddr + c1 + h * BK + k0, v);
            tmem_ld16(taddr + c2 + h * BK + k0, w);
            asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
            for (int kk = 0; kk < 16; ++kk) v[kk] += w[kk];
            // columns past a compact tail tile hold no product: the next GEMM's K
            // padding, written as zeros
            const int cb = 64 * ch + h * BK + k0;
#pragma unroll
            for (int kk = 0; kk < 16; ++kk)
              if (cb + kk >= nt) v[kk] = 0.0f;
            const int slice = 4 * t.tn + 2 * ch + h;
            if (slice >= ldc || row_d < 0) continue;
            uint8_t* tile = tile0 + (int64_t)slice * ts;
            // 16-byte stores: k .. k+3 of a row are contiguous in the core-matrix
            // layout, and a warp's 32 rows fill four whole 128-byte lines
            if (single) {
#pragma unroll
              for (int kk = 0; kk < 16; kk += 4)
                *reinterpret_cast<float4*>(tile + core_off(row_d, k0 + kk)) =
                    make_float4(fa * v[kk], fa * v[kk + 1], fa * v[kk + 2], fa * v[kk + 3]);
            } else {
#pragma unroll
              for (int kk = 0; kk < 16; kk += 4) {
                uint4 hi, lo;
                uint32_t* hp = &hi.x;
                uint32_t* lp = &lo.x;
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                  const float x = fa * v[kk + e];
                  hp[e] = tf32_rna(x);
                  lp[e] = tf32_rna(x - __uint_as_float(hp[e]));
                }
                *reinterpret_cast<uint4*>(tile + core_off(row_d, k0 + kk)) = hi;
                *reinterpret_cast<uint4*>(tile + lo_off + core_off(row_d, k0 + kk)) = lo;
              }
            }
          }
          asm volatile("tcgen05.fence::before_thread_sync;");
          mbar_arrive(smem_u32(&acce_bar[b]));
          ++gc;
        }
        continue;
      }
      double acc[64];
#pragma unroll
      for (int j = 0; j < 64; ++j) acc[j] = 0.0;
      int kacc = 0;
      for (int p = t.p0; p < t.p1; ++p) {
        kacc += pairs[p].nks * BK;
        if (!group_ends(kacc, p, t.p1 - 1)) continue;
        kacc = 0;
        const int b = gc & 1;
        if (!mbar_wait(smem_u32(&accf_bar[b]), (gc >> 1) & 1u, deadline, &abort_flag)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t taddr = tmem + ((uint32_t)(q * 32) << 16) + b * ACC_COLS;
        if (cols) {
#pragma unroll
          for (int c0 = 0; c0 < 64; c0 += 8) {
            float v[8], w[8];
            tmem_ld8(taddr + c1 + c0, v);
            tmem_ld8(taddr + c2 + c0, w);
            asm volatile("tcgen05.wait::ld.sync.aligned;");
#pragma unroll
            for (int i = 0; i < 8; ++i) acc[c0 + i] += static_cast<double>(v[i] + w[i]);
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        mbar_arrive(smem_u32(&acce_bar[b]));
        ++gc;
      }
      if (!ok) break;
      if (row < 0 || !cols) continue;  // lanes without a row (M = 64), warps without columns
      if (t.slot >= 0) {
        double* part = partial + (int64_t)t.slot * (BM * BN) + (int64_t)row * BN + c1;
#pragma unroll
        for (int j = 0; j < 64; ++j) part[j] = acc[j];
      } else if (r < task.m) {
        const int n0 = t.tn * BN + c1;
        double* dst = C + task.c_off + (int64_t)r * task.ldc + n0;
#pragma unroll
        for (int j = 0; j < 64; ++j)
          if (n0 + j < task.n) dst[j] += alpha * acc[j];
      }
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && abort_flag) atomicExch(err, 1);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
}

// Pack FP64 blocks into split-TF32 tiles: one CTA per output tile.
__global__ void __launch_bounds__(256) pack_kernel(const DPack* __restrict__ packs, const double* __restrict__ src,
                                                   uint8_t* __restrict__ dst) {
  const DPack pk = packs[blockIdx.x];
  const int rows_t = pk.tile_rows;
  const uint32_t half = (uint32_t)rows_t * BK * 4;  // bytes of one half (hi or lo) of the tile
  uint8_t* tile = dst + pk.dst_off;
  const int r0 = pk.r0, k0 = pk.tk * BK, span = pk.span;
  for (int e = threadIdx.x; e < span * BK; e += blockDim.x) {
    int r, kk;
    if (!pk.trans) {
      r = e / BK;
      kk = e % BK;
    } else {
      kk = e / span;
      r = e % span;
    }
    const int gr = r0 + r, gk = k0 + kk, tr = pk.ro + r;
    double v = 0.0;
    if (gr < pk.rows && gk < pk.k)
      v = pk.trans ? src[pk.src_off + (int64_t)gk * pk.ld + gr] : src[pk.src_off + (int64_t)gr * pk.ld + gk];
    if (pk.fp32) {
      *reinterpret_cast<float*>(tile + core_off(tr, kk)) = static_cast<float>(v);
    } else {
      uint32_t h, l;
      split2(v, h, l);
      *reinterpret_cast<uint32_t*>(tile + core_off(tr, kk)) = h;
      *reinterpret_cast<uint32_t*>(tile + half + core_off(tr, kk)) = l;
    }
  }
}

// Split-K partials of one output tile summed into C: one thread per valid element of
// the tile (tail tiles are mostly padding; threads past the valid ones exit at once),
// its slots summed four at a time into independent accumulators so that four loads are
// in flight; the summation order is fixed.
__global__ void __launch_bounds__(256) gemm_pk_reduce_kernel(const DReduce* __restrict__ red,
                                                             const DGemmTask* __restrict__ tasks, double alpha,
                                                             const double* __restrict__ partial,
                                                             double* __restrict__ C) {
  const DReduce rd = red[blockIdx.x];
  const DGemmTask task = tasks[rd.task];
  const int m0 = rd.tm * BM, n0 = rd.tn * BN;
  const int vm = min(BM, task.m - m0), vn = min(BN, task.n - n0);
  const int e = blockIdx.y * blockDim.x + threadIdx.x;
  if (vm <= 0 || vn <= 0 || e >= vm * vn) return;
  constexpr int64_t SLOT = BM * BN;
  const int r = e / vn, c = e - r * vn;
  const double* __restrict__ p = partial + (int64_t)rd.slot0 * SLOT + r * BN + c;
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  int k = 0;
  for (; k + 4 <= rd.nslot; k += 4) {
    s0 += p[(k + 0) * SLOT];
    s1 += p[(k + 1) * SLOT];
    s2 += p[(k + 2) * SLOT];
    s3 += p[(k + 3) * SLOT];
  }
  for (; k < rd.nslot; ++k) s0 += p[k * SLOT];
  C[task.c_off + (int64_t)(m0 + r) * task.ldc + (n0 + c)] += alpha * ((s0 + s1) + (s2 + s3));
}

}  // namespace

int pk_smem_bytes() { return SMEM_BYTES; }

void launch_gemm_pk(const uint8_t* Apk, const uint8_t* Bpk, double alpha, double* C, uint8_t* Cpk,
                    const DTile* tiles, int ntiles, const DGemmTask* tasks, const DPkPair* pairs, double* partial,
                    int out_packed, int single, int* err, cudaStream_t st, uint64_t timeout_ns,
                    const int64_t* row_map) {
  if (ntiles <= 0) return;
  static int nsm = 0;
  if (nsm == 0) {
    cudaFuncSetAttribute(gemm_pk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BYTES);
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (nsm <= 0) nsm = 152;
  }
  // one persistent CTA per SM; the bound covers the whole launch, not one tile
  const int grid = ntiles < nsm ? ntiles : nsm;
  gemm_pk_kernel<<<grid, NTHREADS, SMEM_BYTES, st>>>(Apk, Bpk, alpha, C, Cpk, tiles, ntiles, tasks, pairs, partial,
                                                     out_packed, single, err, timeout_ns, row_map);
}

void launch_pack(const DPack* packs, int npacks, const double* src, uint8_t* dst, cudaStream_t st) {
  if (npacks <= 0) return;
  pack_kernel<<<npacks, 256, 0, st>>>(packs, src, dst);
}

void launch_gemm_pk_reduce(const DReduce* red, int nred, const DGemmTask* tasks, double alpha, const double* partial,
                           double* C, cudaStream_t st) {
  if (nred <= 0) return;
  gemm_pk_reduce_kernel<<<dim3(nred, (BM * BN) / 256), 256, 0, st>>>(red, tasks, alpha, partial, C);
}

}  // namespace mpsxx
