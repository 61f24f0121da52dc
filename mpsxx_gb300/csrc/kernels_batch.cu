// Level-1 kernels of the batched Davidson: many independent eigenproblems, one
// launch per operation for all of them.  Problem c owns a slice of one arena:
// vector slot s of problem c starts at off[c] + s * n[c] (slots: trial 0..9,
// sigma 10..19, residual 20, diagonal 21, H_eff*psi input 22 and output 23).
// Every reduction runs over a fixed number of blocks per problem, summed in a fixed
// order, so results do not depend on scheduling.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.hpp"

namespace mpsxx {
namespace {

constexpr int kBt = 256;

__device__ inline double* vslot(double* A, const DBatchProb& p, int s) { return A + p.off + (int64_t)s * p.n; }

// block-wide sums of NV values per thread, thread 0 gets the totals
template <int NV>
__device__ inline void block_sum(double (&v)[NV], double (*red)[NV]) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    double x = v[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][q] = x;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double t = 0.0;
      for (int w = 0; w < kBt / 32; ++w) t += red[w][q];
      v[q] = t;
    }
  }
  __syncthreads();
}

__global__ void bcopy_kernel(const DBatchProb* __restrict__ probs, double* A, int from, int to) {
  const DBatchProb p = probs[blockIdx.y];
  const double* s = vslot(A, p, from);
  double* d = vslot(A, p, to);
  for (int64_t i = blockIdx.x * (int64_t)kBt + threadIdx.x; i < p.n; i += (int64_t)gridDim.x * kBt) d[i] = s[i];
}

__global__ void bzero_kernel(const DBatchProb* __restrict__ probs, double* A, int slot) {
  const DBatchProb p = probs[blockIdx.y];
  double* d = vslot(A, p, slot);
  for (int64_t i = blockIdx.x * (int64_t)kBt + threadIdx.x; i < p.n; i += (int64_t)gridDim.x * kBt) d[i] = 0.0;
}

// partial[c][blk][i*m+j] = sum over the block's chunk of trial_i * sigma_j
__global__ void __launch_bounds__(kBt) bmultidot_partial_kernel(const DBatchProb* __restrict__ probs,
                                                                const double* __restrict__ A, int m,
                                                                double* __restrict__ partial) {
  __shared__ double red[kBt / 32][kMaxDot * kMaxDot];
  const DBatchProb p = probs[blockIdx.y];
  double acc[kMaxDot * kMaxDot];
  const int np = m * m;
  for (int q = 0; q < np; ++q) acc[q] = 0.0;
  const int64_t chunk = (p.n + gridDim.x - 1) / gridDim.x;
  const int64_t lo = blockIdx.x * chunk, hi = min(lo + chunk, p.n);
  const double* T = A + p.off;
  const double* S = A + p.off + 10 * p.n;
  for (int64_t e = lo + threadIdx.x; e < hi; e += kBt) {
    double tv[kMaxDot];
    for (int i = 0; i < m; ++i) tv[i] = T[i * p.n + e];
    for (int j = 0; j < m; ++j) {
      const double sv = S[j * p.n + e];
      for (int i = 0; i < m; ++i) acc[i * m + j] = fma(tv[i], sv, acc[i * m + j]);
    }
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int q = 0; q < np; ++q) {
    double x = acc[q];
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0) red[warp][q] = x;
  }
  __syncthreads();
  if (threadIdx.x < np) {
    double t = 0.0;
    for (int w = 0; w < kBt / 32; ++w) t += red[w][threadIdx.x];
    partial[((int64_t)blockIdx.y * gridDim.x + blockIdx.x) * (kMaxDot * kMaxDot) + threadIdx.x] = t;
  }
}

__global__ void bmultidot_final_kernel(const double* __restrict__ partial, int nblk, int m, double* __restrict__ out) {
  const int c = blockIdx.x, q = threadIdx.x;
  if (q >= m * m) return;
  double t = 0.0;
  for (int b = 0; b < nblk; ++b) t += partial[((int64_t)c * nblk + b) * (kMaxDot * kMaxDot) + q];
  out[c * (kMaxDot * kMaxDot) + q] = t;
}

// trial and sigma slots 0..m-1 of problem c <- their combinations with rvec[c]
__global__ void brotate_kernel(const DBatchProb* __restrict__ probs, double* A, int m, const double* __restrict__ R) {
  const DBatchProb p = probs[blockIdx.y];
  const double* r = R + blockIdx.y * (kMaxDot * kMaxDot);
  for (int64_t e = blockIdx.x * (int64_t)kBt + threadIdx.x; e < p.n; e += (int64_t)gridDim.x * kBt) {
#pragma unroll
    for (int half = 0; half < 2; ++half) {
      double* V = A + p.off + (half ? 10 : 0) * p.n;
      double old[kMaxDot];
      for (int i = 0; i < m; ++i) old[i] = V[i * p.n + e];
      for (int j = 0; j < m; ++j) {
        double v = 0.0;
        for (int i = 0; i < m; ++i) v = fma(r[i * m + j], old[i], v);
        V[j * p.n + e] = v;
      }
    }
  }
}

// residual r = sigma_0 - e * trial_0 (slot 20); partial sums of |r|^2
__global__ void bresidual_kernel(const DBatchProb* __restrict__ probs, double* A, const double* __restrict__ eval,
                                 double* __restrict__ partial) {
  __shared__ double red[kBt / 32][1];
  const DBatchProb p = probs[blockIdx.y];
  const double e = eval[blockIdx.y];
  const double* t0 = vslot(A, p, 0);
  const double* s0 = vslot(A, p, 10);
  double* r = vslot(A, p, 20);
  const int64_t chunk = (p.n + gridDim.x - 1) / gridDim.x;
  const int64_t lo = blockIdx.x * chunk, hi = min(lo + chunk, p.n);
  double v[1] = {0.0};
  for (int64_t i = lo + threadIdx.x; i < hi; i += kBt) {
    const double x = s0[i] - e * t0[i];
    r[i] = x;
    v[0] = fma(x, x, v[0]);
  }
  block_sum<1>(v, red);
  if (threadIdx.x == 0) partial[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = v[0];
}

// the reference's preconditioner: r /= (e - diag), |e - diag| floored at 1e-8
__global__ void bprecondition_kernel(const DBatchProb* __restrict__ probs, double* A, const double* __restrict__ eval) {
  const DBatchProb p = probs[blockIdx.y];
  const double e = eval[blockIdx.y];
  double* r = vslot(A, p, 20);
  const double* d = vslot(A, p, 21);
  for (int64_t i = blockIdx.x * (int64_t)kBt + threadIdx.x; i < p.n; i += (int64_t)gridDim.x * kBt) {
    double den = e - d[i];
    if (fabs(den) < 1.0e-8) den = 1.0e-8;
    r[i] /= den;
  }
}

// partial sums of |r|^2 and (when t >= 0) trial_t . r, r = slot rs
__global__ void bnorm_dot_kernel(const DBatchProb* __restrict__ probs, const double* __restrict__ A, int rs, int t,
                                 double* __restrict__ partial) {
  __shared__ double red[kBt / 32][2];
  const DBatchProb p = probs[blockIdx.y];
  const double* r = A + p.off + (int64_t)rs * p.n;
  const double* v = t >= 0 ? A + p.off + (int64_t)t * p.n : nullptr;
  const int64_t chunk = (p.n + gridDim.x - 1) / gridDim.x;
  const int64_t lo = blockIdx.x * chunk, hi = min(lo + chunk, p.n);
  double s[2] = {0.0, 0.0};
  for (int64_t i = lo + threadIdx.x; i < hi; i += kBt) {
    s[0] = fma(r[i], r[i], s[0]);
    if (v) s[1] = fma(v[i], r[i], s[1]);
  }
  block_sum<2>(s, red);
  if (threadIdx.x == 0) {
    const int64_t b = (int64_t)blockIdx.y * gridDim.x + blockIdx.x;
    partial[2 * b] = s[0];
    partial[2 * b + 1] = s[1];
  }
}

// per problem: out[2c] = sum of the nblk partial pairs (fixed order)
__global__ void bsum_pairs_kernel(const double* __restrict__ partial, int nblk, int nprob, double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nprob) return;
  double a = 0.0, b = 0.0;
  for (int k = 0; k < nblk; ++k) {
    a += partial[2 * ((int64_t)c * nblk + k)];
    b += partial[2 * ((int64_t)c * nblk + k) + 1];
  }
  out[2 * c] = a;
  out[2 * c + 1] = b;
}

__global__ void bsum_kernel(const double* __restrict__ partial, int nblk, int nprob, double* __restrict__ out) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= nprob) return;
  double a = 0.0;
  for (int k = 0; k < nblk; ++k) a += partial[(int64_t)c * nblk + k];
  out[c] = a;
}

// r <- (r - d * trial_t) / |r| with (|r|^2, d) from s[2c]; t < 0: r <- r / |r|
__global__ void bproject_kernel(const DBatchProb* __restrict__ probs, double* A, int rs, int t,
                                const double* __restrict__ s) {
  const DBatchProb p = probs[blockIdx.y];
  const double nrm = sqrt(s[2 * blockIdx.y]);
  const double inv = nrm > 0.0 ? 1.0 / nrm : 0.0;
  const double d = s[2 * blockIdx.y + 1] * inv;  // trial_t . (r / |r|)
  double* r = A + p.off + (int64_t)rs * p.n;
  const double* v = t >= 0 ? A + p.off + (int64_t)t * p.n : nullptr;
  for (int64_t i = blockIdx.x * (int64_t)kBt + threadIdx.x; i < p.n; i += (int64_t)gridDim.x * kBt) {
    const double x = r[i] * inv;
    r[i] = v ? x - d * v[i] : x;
  }
}

int grid_x(int64_t nmax) { return static_cast<int>(std::max<int64_t>(1, std::min<int64_t>((nmax + kBt - 1) / kBt, 64))); }

}  // namespace

void launch_bcopy(const DBatchProb* probs, int nprob, int64_t nmax, double* A, int from, int to, cudaStream_t st) {
  if (nprob <= 0) return;
  bcopy_kernel<<<dim3(grid_x(nmax), nprob), kBt, 0, st>>>(probs, A, from, to);
}

void launch_bzero(const DBatchProb* probs, int nprob, int64_t nmax, double* A, int slot, cudaStream_t st) {
  if (nprob <= 0) return;
  bzero_kernel<<<dim3(grid_x(nmax), nprob), kBt, 0, st>>>(probs, A, slot);
}

void launch_bmultidot(const DBatchProb* probs, int nprob, const double* A, int m, double* partial, double* out,
                      cudaStream_t st) {
  if (nprob <= 0) return;
  bmultidot_partial_kernel<<<dim3(kBatchBlocks, nprob), kBt, 0, st>>>(probs, A, m, partial);
  bmultidot_final_kernel<<<nprob, 128, 0, st>>>(partial, kBatchBlocks, m, out);
}

void launch_brotate(const DBatchProb* probs, int nprob, int64_t nmax, double* A, int m, const double* R,
                    cudaStream_t st) {
  if (nprob <= 0) return;
  brotate_kernel<<<dim3(grid_x(nmax), nprob), kBt, 0, st>>>(probs, A, m, R);
}

void launch_bresidual(const DBatchProb* probs, int nprob, double* A, const double* eval, double* partial,
                      double* rnorm, cudaStream_t st) {
  if (nprob <= 0) return;
  bresidual_kernel<<<dim3(kBatchBlocks, nprob), kBt, 0, st>>>(probs, A, eval, partial);
  bsum_kernel<<<(nprob + 127) / 128, 128, 0, st>>>(partial, kBatchBlocks, nprob, rnorm);
}

void launch_bprecondition(const DBatchProb* probs, int nprob, int64_t nmax, double* A, const double* eval,
                          cudaStream_t st) {
  if (nprob <= 0) return;
  bprecondition_kernel<<<dim3(grid_x(nmax), nprob), kBt, 0, st>>>(probs, A, eval);
}

void launch_bproject(const DBatchProb* probs, int nprob, int64_t nmax, double* A, int rs, int t, double* partial,
                     double* sums, cudaStream_t st) {
  if (nprob <= 0) return;
  bnorm_dot_kernel<<<dim3(kBatchBlocks, nprob), kBt, 0, st>>>(probs, A, rs, t, partial);
  bsum_pairs_kernel<<<(nprob + 127) / 128, 128, 0, st>>>(partial, kBatchBlocks, nprob, sums);
  bproject_kernel<<<dim3(grid_x(nmax), nprob), kBt, 0, st>>>(probs, A, rs, t, sums);
}

}  // namespace mpsxx
