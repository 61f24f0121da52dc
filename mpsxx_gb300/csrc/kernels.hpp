// Device work descriptors and kernel launchers (sm_103a).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace mpsxx {

// One C block of a grouped block GEMM: C[m x n] (ldc) += alpha * sum_p op(A_p) op(B_p).
struct DGemmTask {
  int64_t c_off;
  int m, n, ldc;
  int p0, p1;  // pair range
};
// One (A, B) pair: op(A) is m x k, op(B) is k x n; lda/ldb are the stored row strides.
struct DGemmPair {
  int64_t a_off, b_off;
  int k, lda, ldb, pad;
};
// One output tile of a task over the pair range [p0, p1).  slot < 0: the tile
// adds its result into C; slot >= 0: it writes a 64x64 partial that a fixed-order
// reduction adds into C (split-K for tasks with long pair lists).
struct DTile {
  int task, tm, tn, p0, p1, slot;
  int h64;  // tensor-core tiles: the A rows are a block's 64-row tail tile (see tail64)
  int nt;   // tensor-core tiles: B rows (output columns) of the tile, 128 or a block's
            // compact tail (see tail_cols)
};
// Reduction of the split partials of one output tile.
struct DReduce {
  int task, tm, tn, slot0, nslot, pad;
};

// One block of a batched Jacobi SVD: row-major m x n at src; outputs (offsets into the
// output buffer) U (row-major m x k), s (k) and V^T (row-major k x n), k = min(m, n),
// descending s.
struct DSvdBlock {
  const double* src;
  int64_t u_off, s_off, v_off;
  int m, n, info_slot, pad;
};
constexpr int kJacobiMaxCols = 128;                  // min(m, n) limit of the Jacobi kernel
constexpr size_t kJacobiMaxSmem = 200 * 1024;        // its shared-memory limit per block

// One Gram matrix of the batched eigensolver route: P x P (column-major, the block's
// d x d Gram matrix in the leading corner, -1 on the rest of the diagonal) at G +
// g_off, eigenvalues ascending at w.  The k leading eigenvectors go to out: row-major
// d x k (transposed = 0) or k x d (transposed = 1); s_j = sqrt(lambda_j), zero for
// eigenvalues under 64 eps lambda_max.
struct DEigBlock {
  const double* w;
  double* out;
  double* s;
  int64_t g_off;
  int P, d, k, transposed;
};

// Dense 2-D block copy: dst[r*dld + c] (+)= scale * src[r*sld + c].
struct DCopy {
  int64_t dst_off, src_off;
  int rows, cols, dld, sld;
  double scale;
};
// Destination of a scatter-accumulate: sum over its sources in fixed order.
struct DScatterDst {
  int64_t dst_off;
  int rows, cols, dld, s0, s1, pad;
};
struct DScatterSrc {
  int64_t src_off;
  int sld, pad;
  double coef;
};
// Diagonal task: out block [m x n] (ld n) += sum_p L_p[a*(m+1)] * R_p[b*(n+1)].
struct DDiagTask {
  int64_t out_off;
  int m, n, p0, p1;
};
struct DDiagPair {
  int64_t l_off, r_off;
};
// Noise block of make_noise: y[off + j] += noise * seq[j] for j < n.
struct DNoise {
  int64_t off, n;
};

// Davidson subspace size: multi-dot and rotation kernels handle up to 10 vectors
constexpr int kMaxDot = 10;
// Most CTAs of one multi-dot (each writes kMaxDot * kMaxDot partial sums)
constexpr int kMultidotMaxBlocks = 304;

// One problem of the batched Davidson: its slice of the vector arena.
struct DBatchProb {
  int64_t off, n;
};
constexpr int kBatchBlocks = 16;  // blocks per problem in the batched reductions

constexpr int kGemmTile = 64;
// tensor-core (split TF32) tile: 128 rows x 128 columns (64 on a block's tail)
constexpr int kTcTileM = 128;
constexpr int kTcTileN = 128;

// ---- pre-packed split-TF32 operands -----------------------------------------
// A block of `rows` rows used as a tensor-core operand (A: rows of the result, B: its
// columns) is cut into 128-row tiles; a last tile whose rows fit in 64 is a 64-row tile
// instead (packed compact, half the bytes; M = 64 or N = 64 MMAs): row tile tm of the
// block is such a tile when this holds.
__host__ __device__ constexpr bool tail64(int rows, int tm) {
  return rows % 128 != 0 && rows % 128 <= 64 && tm == rows / 128;
}
// B operands (the result's columns) are cut into 128-row tiles and a compact last
// tile of the remaining rows rounded up to 16 (the N granularity of an M = 128 MMA):
// the number of B rows of column tile tn.
__host__ __device__ constexpr int tail_cols(int rows, int tn) {
  return (tn == rows / 128 && rows % 128 != 0) ? (rows % 128 + 15) / 16 * 16 : 128;
}
constexpr int kPkTileK = 32;                          // K elements per packed slice
// a tile's block pairs accumulate in FP32 (tensor memory) until their padded K reaches
// this, then the group is added into FP64
constexpr int kFlushK = 1024;
constexpr uint32_t kPkTileABytes = 128 * 32 * 4 * 2;  // A tile: hi|lo TF32, 128 rows
constexpr uint32_t kPkTileA1Bytes = 128 * 32 * 4;     // A tile as FP32 values, split on chip
// launch_gemm_pk outputs: FP64 C (or split-K partials), packed hi|lo A tiles, packed
// FP32 A tiles (the next GEMM splits them in shared memory)
constexpr int kOutFP64 = 0, kOutPackedSplit = 1, kOutPackedSingle = 2;
constexpr uint32_t kPkTileBBytes = 128 * 32 * 4 * 2;  // B tile: hi|lo TF32, 128 rows
constexpr uint32_t kPkTileB1Bytes = 128 * 32 * 4;     // B tile as FP32 values, split on chip
// operand formats of launch_gemm_pk (bit mask): FP32 A tiles, FP32 B tiles
constexpr int kSingleA = 1, kSingleB = 2;

// One (A, B) pair over packed operands: byte offsets of the blocks' tile grids.
struct DPkPair {
  int64_t a_pk, b_pk;
  int nks, pad;
};
// One packed tile to produce: element (r, k) of the block is src[src_off + r*ld + k]
// (trans = 0) or src[src_off + k*ld + r] (trans = 1).
// fp32: the tile holds FP32 values (split into hi|lo on chip by the GEMM) instead of
// its hi|lo TF32 halves.  tile_rows: the tile's rows (128, or a compact tail).  The
// pack covers tile rows [ro, ro + span) with block rows r0, r0 + 1, ... (zeros past the
// block's last row): one pack per tile, or several when blocks are stacked in a tile.
struct DPack {
  int64_t src_off, dst_off;
  int rows, k, ld, trans, tile_rows, r0, tk, fp32, ro, span;
};

// out_packed (kOut*): C is written as packed A tiles of the next GEMM (c_off = byte
// offset of the block's grid, ldc = its K slices per row tile) instead of FP64 C /
// partials.  single (kSingleA | kSingleB): the A (B) tiles are FP32 (kPkTileA1Bytes,
// kPkTileB1Bytes each), split into hi|lo in shared memory before the MMAs; otherwise
// packed hi|lo (kPkTileABytes, kPkTileBBytes).
// Every wait of the kernel gives up after timeout_ns (the whole launch): the kernel then
// drains its own bulk copies and MMAs, frees its tensor memory, sets *err and returns.
constexpr uint64_t kPkTimeoutNs = 20000000000ull;  // 20 s
// row_map (packed output only, may be null): the A tiles stack several blocks' rows (a
// stacked panel; the pair's pad field is the panel's first entry in row_map); entry
// (task << 32 | block row) per panel row, -1 for padding rows, says which output block
// and row each tile row is written to.
void launch_gemm_pk(const uint8_t* Apk, const uint8_t* Bpk, double alpha, double* C, uint8_t* Cpk,
                    const DTile* tiles, int ntiles, const DGemmTask* tasks, const DPkPair* pairs, double* partial,
                    int out_packed, int single, int* err, cudaStream_t st, uint64_t timeout_ns = kPkTimeoutNs,
                    const int64_t* row_map = nullptr);
void launch_gemm_pk_reduce(const DReduce* red, int nred, const DGemmTask* tasks, double alpha, const double* partial,
                           double* C, cudaStream_t st);
void launch_pack(const DPack* packs, int npacks, const double* src, uint8_t* dst, cudaStream_t st);
int pk_smem_bytes();

void launch_gemm_f64(int transa, int transb, double alpha, const double* A, const double* B, double* C,
                     const DTile* tiles, int ntiles, const DGemmTask* tasks, const DGemmPair* pairs,
                     double* partial, cudaStream_t st);
void launch_gemm_reduce(const DReduce* red, int nred, const DGemmTask* tasks, double alpha, const double* partial,
                        double* C, cudaStream_t st);
void launch_copy(const DCopy* tasks, int ntasks, const double* src, double* dst, int accumulate,
                 cudaStream_t st);
void launch_scatter(const DScatterDst* dsts, int ndst, const DScatterSrc* srcs, const double* src, double* dst,
                    cudaStream_t st);
// Batched Davidson level-1 operations over problems[0..nprob) (see kernels_batch.cu
// for the slot layout); nmax = the largest problem size; partial holds
// nprob * kBatchBlocks * 100 doubles.
void launch_bcopy(const DBatchProb* probs, int nprob, int64_t nmax, double* A, int from, int to, cudaStream_t st);
void launch_bzero(const DBatchProb* probs, int nprob, int64_t nmax, double* A, int slot, cudaStream_t st);
void launch_bmultidot(const DBatchProb* probs, int nprob, const double* A, int m, double* partial, double* out,
                      cudaStream_t st);
void launch_brotate(const DBatchProb* probs, int nprob, int64_t nmax, double* A, int m, const double* R,
                    cudaStream_t st);
void launch_bresidual(const DBatchProb* probs, int nprob, double* A, const double* eval, double* partial,
                      double* rnorm, cudaStream_t st);
void launch_bprecondition(const DBatchProb* probs, int nprob, int64_t nmax, double* A, const double* eval,
                          cudaStream_t st);
// r = slot rs: r <- (r/|r| - (trial_t . r/|r|) trial_t), or r <- r/|r| when t < 0
void launch_bproject(const DBatchProb* probs, int nprob, int64_t nmax, double* A, int rs, int t, double* partial,
                     double* sums, cudaStream_t st);
// Batched one-sided Jacobi SVD (kernels_svd.cu); smem_bytes >= jacobi_svd_smem of
// every block; info[info_slot] = 1 when a block did not converge.
size_t jacobi_svd_smem(int m, int n);
// -1 on the padded diagonal (indices d..P-1) of every Gram matrix (G zeroed before)
void launch_gram_pad(const DEigBlock* blocks, int nblocks, double* G, cudaStream_t st);
// leading eigenvectors and singular values of every Gram matrix (DEigBlock)
void launch_eig_factors_batched(const DEigBlock* blocks, int nblocks, const double* G, cudaStream_t st);
void launch_jacobi_svd(const DSvdBlock* blocks, int nblocks, size_t smem_bytes, double* out, int* info,
                       cudaStream_t st);
// Eigenvectors G (d x d, column-major, eigenvalues w ascending) of a Gram matrix ->
// the k leading ones in descending order: out (row-major d x k, or its transpose
// k x d when transposed != 0), xcm (column-major d x k) and s_j = sqrt(w) with
// eigenvalues under 64 eps * w_max set to zero.
void launch_eig_factors(const double* G, const double* w, int d, int k, int transposed, double* out, double* xcm,
                        double* s, cudaStream_t st);
// Adjoint of launch_scatter: for every source record s of destination d,
// g[s] = sum_{r,c} Y[d.dst_off + r*d.dld + c] * src[s.src_off + r*s.sld + c]
// (destinations with dst_off < 0 are skipped and leave their g untouched).
void launch_adjoint_scatter(const DScatterDst* dsts, int ndst, const DScatterSrc* srcs, const double* Y,
                            const double* src, double* g, cudaStream_t st);
// G[e] = sum_{k = ptr[e]}^{ptr[e+1]-1} g[idx[k]], summed in index order.
void launch_segment_sum(const int* ptr, const int* idx, const double* g, int ne, double* G, cudaStream_t st);
void launch_diag(const DDiagTask* tasks, int ntasks, const DDiagPair* pairs, const double* L, const double* R,
                 double* out, int max_tiles, cudaStream_t st);

// Level-1 over dense vectors of length n (the block layout of a wavefunction).
void launch_fill(double* x, int64_t n, double v, cudaStream_t st);
void launch_scal_dev(double* x, int64_t n, const double* s, int mode, cudaStream_t st);
void launch_axpy_dev(double* y, const double* x, int64_t n, const double* s, double sign, cudaStream_t st);
void launch_axpy(double* y, const double* x, int64_t n, double a, cudaStream_t st);
void launch_copy_vec(double* y, const double* x, int64_t n, cudaStream_t st);
// y[b.off + j] = y[b.off + j] + noise * seq[j] for every block b (product and sum
// rounded separately, as y + noise*x in double arithmetic without contraction)
void launch_noise_axpy(const DNoise* blocks, int nblocks, const double* seq, double noise, double* y,
                       cudaStream_t st);
// out[i*m + j] = dot(X_i, Y_j) for i < nx, j < ny (vectors strided by `stride`)
void launch_multidot(const double* X, int nx, const double* Y, int ny, int64_t n, int64_t stride, double* out,
                     double* partial, int nblocks, cudaStream_t st);
// new_j = sum_i R[i*ld + j] * old_i, j < m (in place via scratch `tmp` of m*n)
void launch_rotate(double* V, int m, int64_t n, int64_t stride, const double* R, int ldr, double* tmp,
                   cudaStream_t st);
// y -= sum_{i < m} c[i] X[i * stride : i * stride + n], c (m values) on the device
void launch_project_out(double* y, const double* X, int m, int64_t n, int64_t stride, const double* c,
                        cudaStream_t st);
void launch_precondition(double* r, const double* diag, int64_t n, double e, cudaStream_t st);
void launch_scale_blocks_rows(double* data, const int64_t* off, const int* rows, const int* cols,
                              const int64_t* s_off, int nb, const double* s, cudaStream_t st);
void launch_scale_blocks_cols(double* data, const int64_t* off, const int* rows, const int* cols,
                              const int64_t* s_off, int nb, const double* s, cudaStream_t st);
void launch_transpose(const double* src, double* dst, int rows, int cols, cudaStream_t st);

int multidot_blocks(int64_t n);

}  // namespace mpsxx
