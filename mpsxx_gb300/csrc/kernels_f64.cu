// FP64 kernels of the two-site hot path: grouped block GEMM, block copies,
// merged-operator scatter, H_eff diagonal, and the Davidson level-1 operations.
//
// GB300 (sm_103a) has a very small FP64 pipe, so the FP64 path is FMA-bound on
// CUDA cores: a 64x64 output tile per 256-thread CTA, 4x4 register micro-tiles,
// operands staged through shared memory in 16-deep K slices; warps own bands of the
// tile shaped per tile to its valid extent, and bands outside a ragged block skip
// their FMAs.  Every output tile
// is owned by exactly one CTA and its (A,B) pairs are accumulated in enumeration
// order, so results are deterministic run to run.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.hpp"

namespace mpsxx {

namespace {

constexpr int TM = kGemmTile;
constexpr int TN = kGemmTile;
constexpr int TK = 16;

__global__ void __launch_bounds__(256, 2) gemm_f64_kernel(int transa, int transb, double alpha,
                                                       const double* __restrict__ A, const double* __restrict__ B,
                                                       double* __restrict__ C, const DTile* __restrict__ tiles,
                                                       const DGemmTask* __restrict__ tasks,
                                                       const DGemmPair* __restrict__ pairs,
                                                       double* __restrict__ partial) {
  __shared__ double As[TK][TM + 1];
  __shared__ double Bs[TK][TN + 1];
  const DTile t = tiles[blockIdx.x];
  const DGemmTask task = tasks[t.task];
  const int m0 = t.tm * TM, n0 = t.tn * TN;
  // Each warp owns a band of 4 LR rows x 128 / LR columns of the tile: its lanes form
  // an LR x (32 / LR) grid of 4x4 micro-tiles with rows strided by LR and columns by
  // 32 / LR; the 8 bands tile the 64x64 output.  LR (2, 4, 8 or 16) is chosen per tile
  // so that the bands touching the block's valid rows x columns cover the least area,
  // and bands wholly outside skip their FMAs: a ragged block's narrow last tiles (64
  // rows x 6 columns, say) take one band shaped like them instead of several 16 x 32
  // bands, so the FP64 pipe, GB300's narrowest, does little beyond the useful work.
  // The band shape changes which lane computes an element, not its summation order.
  const int vm = min(TM, task.m - m0), vn = min(TN, task.n - n0);
  int LR = 4, best = 1 << 30;
  for (int lr : {4, 2, 8, 16}) {
    const int bh = 4 * lr, bw = 128 / lr;
    const int area = ((vm + bh - 1) / bh) * bh * (((vn + bw - 1) / bw) * bw);
    if (area < best) {
      best = area;
      LR = lr;
    }
  }
  const int LC = 32 / LR;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wr = warp / (LR / 2), wc = warp % (LR / 2);
  const int rb = wr * 4 * LR, cb = wc * (128 / LR);
  const int ty = lane / LC, tx = lane % LC;
  const bool live = (m0 + rb < task.m) && (n0 + cb < task.n);
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  for (int p = t.p0; p < t.p1; ++p) {
    const DGemmPair pr = pairs[p];
    for (int k0 = 0; k0 < pr.k; k0 += TK) {
      for (int e = threadIdx.x; e < TM * TK; e += 256) {
        int r, kk;
        if (!transa) {
          r = e / TK;
          kk = e % TK;
        } else {
          kk = e / TM;
          r = e % TM;
        }
        const int gr = m0 + r, gk = k0 + kk;
        double v = 0.0;
        if (gr < task.m && gk < pr.k)
          v = transa ? A[pr.a_off + (int64_t)gk * pr.lda + gr] : A[pr.a_off + (int64_t)gr * pr.lda + gk];
        As[kk][r] = v;
      }
      for (int e = threadIdx.x; e < TN * TK; e += 256) {
        int c, kk;
        if (!transb) {
          kk = e / TN;
          c = e % TN;
        } else {
          c = e / TK;
          kk = e % TK;
        }
        const int gc = n0 + c, gk = k0 + kk;
        double v = 0.0;
        if (gc < task.n && gk < pr.k)
          v = transb ? B[pr.b_off + (int64_t)gc * pr.ldb + gk] : B[pr.b_off + (int64_t)gk * pr.ldb + gc];
        Bs[kk][c] = v;
      }
      __syncthreads();
      if (live) {
        const int kn = pr.k - k0 < TK ? pr.k - k0 : TK;  // zero-padded K steps are skipped too
        if (kn == TK) {
#pragma unroll
          for (int kk = 0; kk < TK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][rb + ty + LR * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][cb + tx + LC * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
          }
        } else {
          for (int kk = 0; kk < kn; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][rb + ty + LR * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][cb + tx + LC * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
              for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
          }
        }
      }
      __syncthreads();
    }
  }
  if (t.slot >= 0) {
    // split-K partial: the full 64x64 tile, reduced later in chunk order
    double* part = partial + (int64_t)t.slot * (TM * TN);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) part[(rb + ty + LR * i) * TN + cb + tx + LC * j] = acc[i][j];
    return;
  }
  if (!live) return;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int r = m0 + rb + ty + LR * i;
    if (r >= task.m) continue;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int c = n0 + cb + tx + LC * j;
      if (c >= task.n) continue;
      double* dst = C + task.c_off + (int64_t)r * task.ldc + c;
      *dst += alpha * acc[i][j];
    }
  }
}

__global__ void __launch_bounds__(256) gemm_reduce_kernel(const DReduce* __restrict__ red,
                                                          const DGemmTask* __restrict__ tasks, double alpha,
                                                          const double* __restrict__ partial,
                                                          double* __restrict__ C) {
  const DReduce rd = red[blockIdx.x];
  const DGemmTask task = tasks[rd.task];
  const int m0 = rd.tm * TM, n0 = rd.tn * TN;
  for (int e = threadIdx.x; e < TM * TN; e += blockDim.x) {
    const int r = m0 + e / TN, c = n0 + e % TN;
    if (r >= task.m || c >= task.n) continue;
    double s = 0.0;
    for (int k = 0; k < rd.nslot; ++k) s += partial[(int64_t)(rd.slot0 + k) * (TM * TN) + e];
    C[task.c_off + (int64_t)r * task.ldc + c] += alpha * s;
  }
}

__global__ void copy_kernel(const DCopy* __restrict__ tasks, const double* __restrict__ src,
                            double* __restrict__ dst, int accumulate) {
  const DCopy t = tasks[blockIdx.x];
  const int64_t n = (int64_t)t.rows * t.cols;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    const int r = static_cast<int>(e / t.cols), c = static_cast<int>(e % t.cols);
    const double v = t.scale * src[t.src_off + (int64_t)r * t.sld + c];
    double* d = dst + t.dst_off + (int64_t)r * t.dld + c;
    if (accumulate)
      *d += v;
    else
      *d = v;
  }
}

__global__ void scatter_kernel(const DScatterDst* __restrict__ dsts, const DScatterSrc* __restrict__ srcs,
                               const double* __restrict__ src, double* __restrict__ dst) {
  const DScatterDst t = dsts[blockIdx.x];
  const int64_t n = (int64_t)t.rows * t.cols;
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
    const int r = static_cast<int>(e / t.cols), c = static_cast<int>(e % t.cols);
    double acc = 0.0;
    for (int s = t.s0; s < t.s1; ++s) {
      const DScatterSrc q = srcs[s];
      acc = fma(q.coef, src[q.src_off + (int64_t)r * q.sld + c], acc);
    }
    dst[t.dst_off + (int64_t)r * t.dld + c] += acc;
  }
}

// One CTA per destination sub-block; for each of its sources a block-wide dot
// product with a fixed reduction tree (warp shuffles, then the warp totals in order).
__global__ void adjoint_scatter_kernel(const DScatterDst* __restrict__ dsts, const DScatterSrc* __restrict__ srcs,
                                       const double* __restrict__ Y, const double* __restrict__ src,
                                       double* __restrict__ g) {
  __shared__ double warp_part[8];
  const DScatterDst t = dsts[blockIdx.x];
  if (t.dst_off < 0) return;
  const int64_t n = (int64_t)t.rows * t.cols;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int s = t.s0; s < t.s1; ++s) {
    const DScatterSrc q = srcs[s];
    double acc = 0.0;
    for (int64_t e = threadIdx.x; e < n; e += blockDim.x) {
      const int r = static_cast<int>(e / t.cols), c = static_cast<int>(e % t.cols);
      acc = fma(Y[t.dst_off + (int64_t)r * t.dld + c], src[q.src_off + (int64_t)r * q.sld + c], acc);
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) warp_part[warp] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.0;
      for (int w = 0; w < nwarps; ++w) tot += warp_part[w];
      g[s] = tot;
    }
    __syncthreads();
  }
}

__global__ void eig_factors_kernel(const double* __restrict__ G, const double* __restrict__ w, int d, int k,
                                   int transposed, double* __restrict__ out, double* __restrict__ xcm,
                                   double* __restrict__ s) {
  const int64_t n = (int64_t)d * k;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    const int r = static_cast<int>(e % d), j = static_cast<int>(e / d);
    const double v = G[r + (int64_t)(d - 1 - j) * d];
    xcm[r + (int64_t)j * d] = v;
    if (transposed)
      out[(int64_t)j * d + r] = v;
    else
      out[(int64_t)r * k + j] = v;
    if (r == 0) {
      const double lam = w[d - 1 - j], top = w[d - 1];
      s[j] = lam > 64.0 * 2.220446049250313e-16 * top ? sqrt(lam) : 0.0;
    }
  }
}

__global__ void segment_sum_kernel(const int* __restrict__ ptr, const int* __restrict__ idx,
                                   const double* __restrict__ g, int ne, double* __restrict__ G) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  double acc = 0.0;
  for (int k = ptr[e]; k < ptr[e + 1]; ++k) acc += g[idx[k]];
  G[e] = acc;
}

// diag[a, b] += sum_p L_p[a, a] R_p[b, b] over a block's (L, R) pairs, one CTA per
// 32 x 32 tile of the block (blockIdx.y); the tied diagonals of 32 pairs at a time are
// gathered into shared memory, each thread sums four outputs over the pairs in order.
constexpr int kDiagTile = 32, kDiagPairs = 32;
__global__ void __launch_bounds__(256) diag_kernel(const DDiagTask* __restrict__ tasks,
                                                   const DDiagPair* __restrict__ pairs, const double* __restrict__ L,
                                                   const double* __restrict__ R, double* __restrict__ out) {
  __shared__ double ls[kDiagPairs][kDiagTile];
  __shared__ double rs[kDiagPairs][kDiagTile];
  const DDiagTask t = tasks[blockIdx.x];
  const int tcols = (t.n + kDiagTile - 1) / kDiagTile;
  const int ntile = ((t.m + kDiagTile - 1) / kDiagTile) * tcols;
  if ((int)blockIdx.y >= ntile) return;
  const int a0 = (blockIdx.y / tcols) * kDiagTile, b0 = (blockIdx.y % tcols) * kDiagTile;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // column tx, rows ty + 8 i
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  for (int p0 = t.p0; p0 < t.p1; p0 += kDiagPairs) {
    const int np = t.p1 - p0 < kDiagPairs ? t.p1 - p0 : kDiagPairs;
    __syncthreads();
    for (int e = threadIdx.x; e < np * kDiagTile; e += blockDim.x) {
      const int q = e / kDiagTile, i = e % kDiagTile;
      const DDiagPair pr = pairs[p0 + q];
      const int a = a0 + i, b = b0 + i;
      ls[q][i] = a < t.m ? L[pr.l_off + (int64_t)a * (t.m + 1)] : 0.0;
      rs[q][i] = b < t.n ? R[pr.r_off + (int64_t)b * (t.n + 1)] : 0.0;
    }
    __syncthreads();
    for (int q = 0; q < np; ++q) {
      const double r = rs[q][tx];
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[i] = fma(ls[q][ty + 8 * i], r, acc[i]);
    }
  }
  const int b = b0 + tx;
  if (b >= t.n) return;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const int a = a0 + ty + 8 * i;
    if (a < t.m) out[t.out_off + (int64_t)a * t.n + b] += acc[i];
  }
}

__global__ void fill_kernel(double* x, int64_t n, double v) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] = v;
}

// mode 0: x *= s[0]; mode 1: x *= 1/sqrt(s[0]) (s holds a squared norm)
__global__ void scal_dev_kernel(double* x, int64_t n, const double* s, int mode) {
  const double f = mode == 0 ? s[0] : 1.0 / sqrt(s[0]);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    x[i] *= f;
}

__global__ void axpy_dev_kernel(double* y, const double* x, int64_t n, const double* s, double sign) {
  const double a = sign * s[0];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = fma(a, x[i], y[i]);
}

__global__ void axpy_kernel(double* y, const double* x, int64_t n, double a) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = fma(a, x[i], y[i]);
}

__global__ void noise_axpy_kernel(const DNoise* __restrict__ blocks, const double* __restrict__ seq, double noise,
                                  double* __restrict__ y) {
  const DNoise b = blocks[blockIdx.x];
  for (int64_t j = threadIdx.x; j < b.n; j += blockDim.x)
    y[b.off + j] = __dadd_rn(y[b.off + j], __dmul_rn(noise, seq[j]));
}

__global__ void copy_vec_kernel(double* y, const double* x, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    y[i] = x[i];
}


// Each CTA reduces a contiguous chunk into partial[blk][i*ny+j]; a fixed-order
// second pass makes the sum deterministic.  The chunk is walked in tiles of
// kDotTile elements staged in shared memory (all nx + ny vectors, coalesced loads);
// each of the nx*ny products is owned by g = 256 / (nx*ny) threads that sum fixed
// strided parts of the tile in registers, and the g partial sums of a product are
// added in thread order at the end — no per-thread arrays indexed at run time.
constexpr int kDotTile = 128;
__global__ void __launch_bounds__(256) multidot_partial_kernel(const double* __restrict__ X, int nx,
                                                               const double* __restrict__ Y, int ny, int64_t n,
                                                               int64_t stride, double* __restrict__ partial) {
  __shared__ double xs[kMaxDot][kDotTile];
  __shared__ double ys[kMaxDot][kDotTile];
  __shared__ double red[256];
  const int np = nx * ny;
  const int g = 256 / np;  // threads per product (>= 2 for np <= 100)
  const int t = threadIdx.x;
  const int q = t / g, sub = t % g;
  const bool active = q < np;
  const int qi = active ? q / ny : 0, qj = active ? q % ny : 0;
  double acc = 0.0;
  const int64_t chunk = (n + gridDim.x - 1) / gridDim.x;
  const int64_t lo = blockIdx.x * chunk;
  const int64_t hi = lo + chunk < n ? lo + chunk : n;
  for (int64_t e0 = lo; e0 < hi; e0 += kDotTile) {
    const int len = hi - e0 < kDotTile ? static_cast<int>(hi - e0) : kDotTile;
    __syncthreads();  // the previous tile is consumed
    for (int v = 0; v < nx + ny; ++v) {
      const double* src = v < nx ? X + v * stride : Y + (v - nx) * stride;
      double* dst = v < nx ? xs[v] : ys[v - nx];
      for (int k = t; k < len; k += 256) dst[k] = src[e0 + k];
    }
    __syncthreads();
    if (active)
      for (int k = sub; k < len; k += g) acc = fma(xs[qi][k], ys[qj][k], acc);
  }
  red[t] = acc;
  __syncthreads();
  if (active && sub == 0) {
    double v = 0.0;
    for (int k = 0; k < g; ++k) v += red[t + k];
    partial[blockIdx.x * (kMaxDot * kMaxDot) + q] = v;
  }
}

__global__ void multidot_final_kernel(const double* __restrict__ partial, int nblocks, int np,
                                      double* __restrict__ out) {
  const int q = threadIdx.x;
  if (q >= np) return;
  double v = 0.0;
  for (int b = 0; b < nblocks; ++b) v += partial[b * (kMaxDot * kMaxDot) + q];
  out[q] = v;
}

// y -= sum_{i < m} c[i] X[:, i] (X's vectors stride apart; c on the device).
__global__ void project_out_kernel(double* __restrict__ y, const double* __restrict__ X, int m, int64_t n,
                                   int64_t stride, const double* __restrict__ c) {
  double cc[kMaxDot];
#pragma unroll
  for (int i = 0; i < kMaxDot; ++i) cc[i] = i < m ? c[i] : 0.0;
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    double v = y[e];
#pragma unroll
    for (int i = 0; i < kMaxDot; ++i)
      if (i < m) v = fma(-cc[i], X[i * stride + e], v);
    y[e] = v;
  }
}

// V[:, j] = sum_i V[:, i] R[i, j] for j < m, in place per element (loops unrolled to
// kMaxDot so that the element's m values stay in registers).
__global__ void rotate_kernel(double* V, int m, int64_t n, int64_t stride, const double* __restrict__ R, int ldr) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
    double old[kMaxDot];
#pragma unroll
    for (int i = 0; i < kMaxDot; ++i) old[i] = i < m ? V[i * stride + e] : 0.0;
#pragma unroll
    for (int j = 0; j < kMaxDot; ++j) {
      if (j < m) {
        double v = 0.0;
#pragma unroll
        for (int i = 0; i < kMaxDot; ++i)
          if (i < m) v = fma(R[i * ldr + j], old[i], v);
        V[j * stride + e] = v;
      }
    }
  }
}

__global__ void precondition_kernel(double* r, const double* __restrict__ diag, int64_t n, double e) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    double denm = e - diag[i];
    if (fabs(denm) < 1.0e-8) denm = 1.0e-8;
    r[i] /= denm;
  }
}

__global__ void scale_rows_kernel(double* data, const int64_t* off, const int* rows, const int* cols,
                                  const int64_t* s_off, const double* s) {
  const int b = blockIdx.x;
  const int64_t n = (int64_t)rows[b] * cols[b];
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) data[off[b] + e] *= s[s_off[b] + e / cols[b]];
}

__global__ void scale_cols_kernel(double* data, const int64_t* off, const int* rows, const int* cols,
                                  const int64_t* s_off, const double* s) {
  const int b = blockIdx.x;
  const int64_t n = (int64_t)rows[b] * cols[b];
  for (int64_t e = threadIdx.x; e < n; e += blockDim.x) data[off[b] + e] *= s[s_off[b] + e % cols[b]];
}

__global__ void transpose_kernel(const double* __restrict__ src, double* __restrict__ dst, int rows, int cols) {
  __shared__ double tile[32][33];
  const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int r = by + j, c = bx + threadIdx.x;
    if (r < rows && c < cols) tile[j][threadIdx.x] = src[(int64_t)r * cols + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += 8) {
    const int r = bx + j, c = by + threadIdx.x;  // dst is cols x rows
    if (r < cols && c < rows) dst[(int64_t)r * rows + c] = tile[threadIdx.x][j];
  }
}

inline int grid_for(int64_t n) {
  int64_t g = (n + 255) / 256;
  if (g > 152 * 16) g = 152 * 16;
  if (g < 1) g = 1;
  return static_cast<int>(g);
}

}  // namespace

void launch_gemm_f64(int transa, int transb, double alpha, const double* A, const double* B, double* C,
                     const DTile* tiles, int ntiles, const DGemmTask* tasks, const DGemmPair* pairs,
                     double* partial, cudaStream_t st) {
  if (ntiles <= 0) return;
  gemm_f64_kernel<<<ntiles, 256, 0, st>>>(transa, transb, alpha, A, B, C, tiles, tasks, pairs, partial);
}

void launch_gemm_reduce(const DReduce* red, int nred, const DGemmTask* tasks, double alpha, const double* partial,
                        double* C, cudaStream_t st) {
  if (nred <= 0) return;
  gemm_reduce_kernel<<<nred, 256, 0, st>>>(red, tasks, alpha, partial, C);
}

void launch_copy(const DCopy* tasks, int ntasks, const double* src, double* dst, int accumulate, cudaStream_t st) {
  if (ntasks <= 0) return;
  copy_kernel<<<ntasks, 256, 0, st>>>(tasks, src, dst, accumulate);
}

void launch_scatter(const DScatterDst* dsts, int ndst, const DScatterSrc* srcs, const double* src, double* dst,
                    cudaStream_t st) {
  if (ndst <= 0) return;
  scatter_kernel<<<ndst, 256, 0, st>>>(dsts, srcs, src, dst);
}

void launch_adjoint_scatter(const DScatterDst* dsts, int ndst, const DScatterSrc* srcs, const double* Y,
                            const double* src, double* g, cudaStream_t st) {
  if (ndst <= 0) return;
  adjoint_scatter_kernel<<<ndst, 256, 0, st>>>(dsts, srcs, Y, src, g);
}

void launch_eig_factors(const double* G, const double* w, int d, int k, int transposed, double* out, double* xcm,
                        double* s, cudaStream_t st) {
  const int64_t n = (int64_t)d * k;
  if (n <= 0) return;
  const int grid = static_cast<int>(std::min<int64_t>((n + 255) / 256, 4096));
  eig_factors_kernel<<<grid, 256, 0, st>>>(G, w, d, k, transposed, out, xcm, s);
}

void launch_segment_sum(const int* ptr, const int* idx, const double* g, int ne, double* G, cudaStream_t st) {
  if (ne <= 0) return;
  segment_sum_kernel<<<(ne + 255) / 256, 256, 0, st>>>(ptr, idx, g, ne, G);
}

void launch_diag(const DDiagTask* tasks, int ntasks, const DDiagPair* pairs, const double* L, const double* R,
                 double* out, int max_tiles, cudaStream_t st) {
  if (ntasks <= 0) return;
  if (max_tiles <= 0) return;
  diag_kernel<<<dim3(ntasks, max_tiles), 256, 0, st>>>(tasks, pairs, L, R, out);
}

void launch_fill(double* x, int64_t n, double v, cudaStream_t st) {
  if (n <= 0) return;
  fill_kernel<<<grid_for(n), 256, 0, st>>>(x, n, v);
}

void launch_scal_dev(double* x, int64_t n, const double* s, int mode, cudaStream_t st) {
  if (n <= 0) return;
  scal_dev_kernel<<<grid_for(n), 256, 0, st>>>(x, n, s, mode);
}

void launch_axpy_dev(double* y, const double* x, int64_t n, const double* s, double sign, cudaStream_t st) {
  if (n <= 0) return;
  axpy_dev_kernel<<<grid_for(n), 256, 0, st>>>(y, x, n, s, sign);
}

void launch_axpy(double* y, const double* x, int64_t n, double a, cudaStream_t st) {
  if (n <= 0) return;
  axpy_kernel<<<grid_for(n), 256, 0, st>>>(y, x, n, a);
}

void launch_noise_axpy(const DNoise* blocks, int nblocks, const double* seq, double noise, double* y,
                       cudaStream_t st) {
  if (nblocks <= 0) return;
  noise_axpy_kernel<<<nblocks, 256, 0, st>>>(blocks, seq, noise, y);
}

void launch_copy_vec(double* y, const double* x, int64_t n, cudaStream_t st) {
  if (n <= 0) return;
  copy_vec_kernel<<<grid_for(n), 256, 0, st>>>(y, x, n);
}

int multidot_blocks(int64_t n) {
  int64_t b = (n + 2047) / 2048;
  if (b > kMultidotMaxBlocks) b = kMultidotMaxBlocks;
  if (b < 1) b = 1;
  return static_cast<int>(b);
}

void launch_multidot(const double* X, int nx, const double* Y, int ny, int64_t n, int64_t stride, double* out,
                     double* partial, int nblocks, cudaStream_t st) {
  multidot_partial_kernel<<<nblocks, 256, 0, st>>>(X, nx, Y, ny, n, stride, partial);
  multidot_final_kernel<<<1, 128, 0, st>>>(partial, nblocks, nx * ny, out);
}

void launch_rotate(double* V, int m, int64_t n, int64_t stride, const double* R, int ldr, double* tmp,
                   cudaStream_t st) {
  (void)tmp;
  if (n <= 0) return;
  rotate_kernel<<<grid_for(n), 256, 0, st>>>(V, m, n, stride, R, ldr);
}

void launch_project_out(double* y, const double* X, int m, int64_t n, int64_t stride, const double* c,
                        cudaStream_t st) {
  if (n <= 0 || m <= 0) return;
  project_out_kernel<<<grid_for(n), 256, 0, st>>>(y, X, m, n, stride, c);
}

void launch_precondition(double* r, const double* diag, int64_t n, double e, cudaStream_t st) {
  if (n <= 0) return;
  precondition_kernel<<<grid_for(n), 256, 0, st>>>(r, diag, n, e);
}

void launch_scale_blocks_rows(double* data, const int64_t* off, const int* rows, const int* cols,
                              const int64_t* s_off, int nb, const double* s, cudaStream_t st) {
  if (nb <= 0) return;
  scale_rows_kernel<<<nb, 256, 0, st>>>(data, off, rows, cols, s_off, s);
}

void launch_scale_blocks_cols(double* data, const int64_t* off, const int* rows, const int* cols,
                              const int64_t* s_off, int nb, const double* s, cudaStream_t st) {
  if (nb <= 0) return;
  scale_cols_kernel<<<nb, 256, 0, st>>>(data, off, rows, cols, s_off, s);
}

void launch_transpose(const double* src, double* dst, int rows, int cols, cudaStream_t st) {
  if (rows <= 0 || cols <= 0) return;
  dim3 grid((cols + 31) / 32, (rows + 31) / 32);
  transpose_kernel<<<grid, dim3(32, 8), 0, st>>>(src, dst, rows, cols);
}

}  // namespace mpsxx
