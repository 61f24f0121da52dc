// Batched one-sided Jacobi SVD (Hestenes) of small dense blocks: one CTA per block,
// the block and its right rotations held in shared memory, every block of a launch
// independent.  FP64 throughout.  For the block-sparse wavefunctions of the sweep the
// sector blocks are mostly far below the sizes where cuSOLVER's gesvd stops being
// latency-bound, and one launch replaces one solver call per block.
//
// Method (Hestenes 1958, with the Rutishauser rotation): orthogonalise the columns of
// W (the block, or its transpose so that W has at most as many columns as rows) by
// plane rotations applied to W and to V = I; a pair (p, q) is rotated when
// |w_p . w_q| > tol * |w_p| |w_q|.  Sweeps visit all pairs in a round-robin
// tournament order (n/2 disjoint pairs per round, one warp per pair) until a sweep
// rotates nothing or kJacobiSweeps sweeps have run.  Then s_j = |w_j|, u_j = w_j / s_j,
// and the triplets are sorted by decreasing s.  Columns that end at or below the
// numerical-zero level (|w_j|^2 <= (rows eps)^2 |A|_F^2) took no part in the
// rotations and are not orthogonal to the others: like LAPACK's gesvd, their u_j are
// replaced by an orthonormal completion (unit vectors e_0, e_1, ... orthogonalised
// twice against the columns before them, the first with a remaining norm above 1/2),
// so both factors are orthonormal whatever the rank; s_j keeps its (tiny) value.  The
// schedule and every reduction are fixed, so results do not depend on timing.
#include <cuda_runtime.h>

#include <cstdint>

#include "kernels.hpp"

namespace mpsxx {
namespace {

constexpr int kJt = 256;
constexpr int kJacobiSweeps = 40;
constexpr double kEps = 2.220446049250313e-16;

__device__ inline double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// the k-th pair (p < q) of round r of a round-robin tournament on n2 (even) players
// (circle method: player n2-1 stays, the others rotate; every pair meets once)
__device__ inline void pair_of(int k, int r, int n2, int* p, int* q) {
  const int m = n2 - 1;
  int a, b;
  if (k == 0) {
    a = r % m;
    b = m;
  } else {
    a = (r + k) % m;
    b = (r - k + m) % m;
  }
  *p = a < b ? a : b;
  *q = a < b ? b : a;
}

__global__ void __launch_bounds__(kJt) jacobi_svd_kernel(const DSvdBlock* __restrict__ blocks,
                                                         double* __restrict__ out, int* __restrict__ info) {
  extern __shared__ double sm[];
  __shared__ int rotated;
  __shared__ int perm[kJacobiMaxCols];
  __shared__ double norm[kJacobiMaxCols];
  __shared__ double wsum[kJt / 32];
  const DSvdBlock b = blocks[blockIdx.x];
  const bool tr = b.n > b.m;          // W = A^T when A is wide
  const int rows = tr ? b.n : b.m;    // rows of W
  const int cols = tr ? b.m : b.n;    // columns of W (<= rows)
  double* W = sm;                     // column-major rows x cols
  double* V = sm + (int64_t)rows * cols;  // column-major cols x cols
  const double* A = b.src;            // row-major m x n
  for (int e = threadIdx.x; e < rows * cols; e += kJt) {
    const int i = e % rows, j = e / rows;
    W[e] = tr ? A[(int64_t)j * b.n + i] : A[(int64_t)i * b.n + j];
  }
  for (int e = threadIdx.x; e < cols * cols; e += kJt) V[e] = (e % cols == e / cols) ? 1.0 : 0.0;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = kJt / 32;
  // |W|_F^2: columns below (rows eps)^2 |W|_F^2 are numerically zero and never rotated
  {
    double f = 0.0;
    for (int e = threadIdx.x; e < rows * cols; e += kJt) {
      const int i = e % rows, j = e / rows;
      const double x = tr ? A[(int64_t)j * b.n + i] : A[(int64_t)i * b.n + j];
      f = fma(x, x, f);
    }
    f = warp_sum(f);
    if (lane == 0) wsum[warp] = f;
  }
  __syncthreads();
  double frob2 = 0.0;
  for (int w = 0; w < nwarp; ++w) frob2 += wsum[w];
  const double tiny = double(rows) * kEps * double(rows) * kEps * frob2;
  const int n2 = cols + (cols & 1);  // even number of players (a dummy when cols is odd)
  int sweep = 0;
  for (; sweep < kJacobiSweeps && cols > 1; ++sweep) {
    if (threadIdx.x == 0) rotated = 0;
    __syncthreads();
    for (int r = 0; r < n2 - 1; ++r) {
      for (int k = warp; k < n2 / 2; k += nwarp) {
        int p, q;
        pair_of(k, r, n2, &p, &q);
        if (q >= cols) continue;  // the dummy player
        double* wp = W + (int64_t)p * rows;
        double* wq = W + (int64_t)q * rows;
        double al = 0.0, be = 0.0, ga = 0.0;
        for (int i = lane; i < rows; i += 32) {
          const double x = wp[i], y = wq[i];
          al = fma(x, x, al);
          be = fma(y, y, be);
          ga = fma(x, y, ga);
        }
        al = warp_sum(al);
        be = warp_sum(be);
        ga = warp_sum(ga);
        if (al <= tiny || be <= tiny || fabs(ga) <= rows * kEps * sqrt(al * be)) continue;
        const double zeta = (be - al) / (2.0 * ga);
        const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
        for (int i = lane; i < rows; i += 32) {
          const double x = wp[i], y = wq[i];
          wp[i] = c * x - s * y;
          wq[i] = s * x + c * y;
        }
        double* vp = V + (int64_t)p * cols;
        double* vq = V + (int64_t)q * cols;
        for (int i = lane; i < cols; i += 32) {
          const double x = vp[i], y = vq[i];
          vp[i] = c * x - s * y;
          vq[i] = s * x + c * y;
        }
        if (lane == 0) rotated = 1;
      }
      __syncthreads();
    }
    const int any = rotated;
    __syncthreads();
    if (!any) break;
  }
  if (threadIdx.x == 0 && info) info[b.info_slot] = (sweep >= kJacobiSweeps && cols > 1) ? 1 : 0;
  // singular values and their descending order (ties keep the column order)
  for (int j = warp; j < cols; j += nwarp) {
    double v = 0.0;
    for (int i = lane; i < rows; i += 32) v = fma(W[(int64_t)j * rows + i], W[(int64_t)j * rows + i], v);
    v = warp_sum(v);
    if (lane == 0) norm[j] = sqrt(v);
  }
  __syncthreads();
  for (int j = threadIdx.x; j < cols; j += kJt) {
    int rank = 0;
    for (int l = 0; l < cols; ++l) rank += (norm[l] > norm[j]) || (norm[l] == norm[j] && l < j);
    perm[rank] = j;
  }
  __syncthreads();
  // normalise the columns; then complete the numerically-zero ones (sorted last) in
  // place, one at a time, against the columns before them in the sorted order
  for (int e = threadIdx.x; e < rows * cols; e += kJt) {
    const int c = e / rows;
    const double s = norm[c];
    if (s * s > tiny && s > 0.0) W[e] /= s;
  }
  __syncthreads();
  if (warp == 0) {  // serial over the columns, reductions within the warp
    for (int j = 0; j < cols; ++j) {
      const int c = perm[j];
      const double s = norm[c];
      if (s * s > tiny && s > 0.0) continue;
      double* wc = W + (int64_t)c * rows;
      for (int cand = 0; cand < rows; ++cand) {
        for (int i = lane; i < rows; i += 32) wc[i] = (i == cand) ? 1.0 : 0.0;
        __syncwarp();
        for (int pass = 0; pass < 2; ++pass) {
          for (int l = 0; l < j; ++l) {
            const double* wl = W + (int64_t)perm[l] * rows;
            double d = 0.0;
            for (int i = lane; i < rows; i += 32) d = fma(wl[i], wc[i], d);
            d = warp_sum(d);
            for (int i = lane; i < rows; i += 32) wc[i] = fma(-d, wl[i], wc[i]);
            __syncwarp();
          }
        }
        double nn = 0.0;
        for (int i = lane; i < rows; i += 32) nn = fma(wc[i], wc[i], nn);
        nn = sqrt(warp_sum(nn));
        if (nn > 0.5) {
          for (int i = lane; i < rows; i += 32) wc[i] /= nn;
          __syncwarp();
          break;
        }
      }
    }
  }
  __syncthreads();
  // outputs: U row-major m x k, s (k), V^T row-major k x n, k = cols
  double* U = out + b.u_off;
  double* S = out + b.s_off;
  double* Vt = out + b.v_off;
  const int k = cols;
  for (int j = threadIdx.x; j < k; j += kJt) S[j] = norm[perm[j]];
  if (!tr) {
    // A = W-basis: U_j = w_perm(j) (normalised, m = rows), V^T[j][c] = V[c][perm(j)]
    for (int e = threadIdx.x; e < b.m * k; e += kJt) {
      const int i = e / k, j = e % k;
      U[e] = W[(int64_t)perm[j] * rows + i];
    }
    for (int e = threadIdx.x; e < k * b.n; e += kJt) {
      const int j = e / b.n, c = e % b.n;
      Vt[e] = V[(int64_t)perm[j] * cols + c];
    }
  } else {
    // A^T = W-basis: A = V S W^T, so U = V (m = cols rows), V^T_j = w_perm(j) (normalised)
    for (int e = threadIdx.x; e < b.m * k; e += kJt) {
      const int i = e / k, j = e % k;
      U[e] = V[(int64_t)perm[j] * cols + i];
    }
    for (int e = threadIdx.x; e < k * b.n; e += kJt) {
      const int j = e / b.n, c = e % b.n;
      Vt[e] = W[(int64_t)perm[j] * rows + c];
    }
  }
}

__global__ void gram_pad_kernel(const DEigBlock* __restrict__ blocks, double* __restrict__ G) {
  const DEigBlock b = blocks[blockIdx.x];
  for (int i = b.d + threadIdx.x; i < b.P; i += blockDim.x) G[b.g_off + (int64_t)i * (b.P + 1)] = -1.0;
}

__global__ void eig_factors_batched_kernel(const DEigBlock* __restrict__ blocks, const double* __restrict__ G) {
  const DEigBlock b = blocks[blockIdx.x];
  const double top = b.w[b.P - 1];
  for (int e = threadIdx.x; e < b.d * b.k; e += blockDim.x) {
    const int r = e % b.d, j = e / b.d;
    const double v = G[b.g_off + r + (int64_t)(b.P - 1 - j) * b.P];
    if (b.transposed)
      b.out[(int64_t)j * b.d + r] = v;
    else
      b.out[(int64_t)r * b.k + j] = v;
  }
  for (int j = threadIdx.x; j < b.k; j += blockDim.x) {
    const double lam = b.w[b.P - 1 - j];
    b.s[j] = lam > 64.0 * kEps * top ? sqrt(lam) : 0.0;
  }
}

}  // namespace

void launch_gram_pad(const DEigBlock* blocks, int nblocks, double* G, cudaStream_t st) {
  if (nblocks <= 0) return;
  gram_pad_kernel<<<nblocks, 128, 0, st>>>(blocks, G);
}

void launch_eig_factors_batched(const DEigBlock* blocks, int nblocks, const double* G, cudaStream_t st) {
  if (nblocks <= 0) return;
  eig_factors_batched_kernel<<<nblocks, 256, 0, st>>>(blocks, G);
}

size_t jacobi_svd_smem(int m, int n) {
  const int rows = m > n ? m : n, cols = m > n ? n : m;
  return (size_t(rows) * cols + size_t(cols) * cols) * sizeof(double);
}

void launch_jacobi_svd(const DSvdBlock* blocks, int nblocks, size_t smem_bytes, double* out, int* info,
                       cudaStream_t st) {
  if (nblocks <= 0) return;
  static size_t configured = 0;
  if (smem_bytes > configured) {
    cudaFuncSetAttribute(jacobi_svd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem_bytes));
    configured = smem_bytes;
  }
  jacobi_svd_kernel<<<nblocks, kJt, smem_bytes, st>>>(blocks, out, info);
}

}  // namespace mpsxx
