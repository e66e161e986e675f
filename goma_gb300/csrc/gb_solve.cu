// Newton linear algebra on the device:
//   row_sum_scale   restates row_sum_scale_MSR (src/sl_matrix_util.c:506)
//   norms           L2_norm / L1_norm / Loo_norm (src/mm_sol_nonlinear.c:3177-3530)
//   SpMV            MV_MSR semantics (src/sl_auxutil.c:373) on the CSR copy
//   ILU(0)          the preconditioner AztecOO builds for "Preconditioner =
//                   ilu" (dom_decomp + subdomain ILU(0), src/sl_util.c:556),
//                   same ordering and pattern; factorised and applied by
//                   node levels (one warp per node, unknowns of a node in
//                   order), the level sequence replayed as a CUDA graph
//   GMRES(m)        right-preconditioned restarted GMRES with classical
//                   Gram-Schmidt + reorthogonalisation (the reference's
//                   "Solution Algorithm = gmres", Krylov size 30,
//                   src/sl_util.c:417) in FP64, or in FP32 inside FP64
//                   iterative refinement
// Reductions use a fixed grid and a fixed combination order, so every
// result is bitwise reproducible run to run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <type_traits>
#include <vector>

#include "gb_context.h"
#include "gb_solve.h"

namespace gb {

static constexpr int kRedBlocks = 304;  // 2 x 152 SMs
static constexpr int kRedThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Arithmetic type of the vector kernels: FP64 data is combined in FP64, FP32
// data in FP32.  On GB300 FP64 arithmetic runs at 1/64 of the FP32 rate, so
// an FP32 kernel that widened its operands to FP64 would be bound by the
// FP64 pipe instead of HBM; the FP32 inner solve gets its accuracy from the
// FP64 refinement around it.
template <class T>
struct AccT {
  using type = double;
};
template <>
struct AccT<float> {
  using type = float;
};
template <class T>
using acc_t = typename AccT<T>::type;
__device__ __forceinline__ double fmx(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float fmx(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double wsum(double v) { return warp_sum(v); }
__device__ __forceinline__ float wsum(float v) { return warp_sumf(v); }

// ------------------------------------------------------------ scaling

__global__ void row_sum_scale_kernel(int N, const int64_t *__restrict__ rowptr,
                                     const int64_t *__restrict__ diag, double *__restrict__ vals,
                                     double *__restrict__ R, double *__restrict__ scale,
                                     int *__restrict__ zero_rows) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (i >= N) return;
  const int64_t r0 = rowptr[i], r1 = rowptr[i + 1];
  double s = 0.0;
  for (int64_t k = r0 + lane; k < r1; k += 32) s += fabs(vals[k]);
  s = warp_sum(s);
  const double d = vals[diag[i]];
  if (fabs(d) > 1.0e-200 && d < 0.0) s = -s;
  if (s == 0.0) {
    if (lane == 0) atomicAdd(zero_rows, 1);
    s = 1.0;
  }
  // one division per row: on GB300 an FP64 division per entry made this
  // kernel FP64-bound (12.7 ms at 308 M entries); the products differ from
  // the quotients by at most one rounding
  const double rs = 1.0 / s;
  for (int64_t k = r0 + lane; k < r1; k += 32) vals[k] = vals[k] * rs;
  if (lane == 0) {
    scale[i] = s;
    R[i] = R[i] / s;
  }
}

// ------------------------------------------------------------ reductions

template <class T>
__global__ void norms_partial_kernel(int N, const T *__restrict__ x, double *__restrict__ part) {
  __shared__ double sh[3][kRedThreads];
  using A = acc_t<T>;
  A s2 = 0, s1 = 0, mx = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const A v = (A)x[i];
    s2 = fmx(v, v, s2);
    s1 += fabs(v);
    mx = fmax(mx, fabs(v));
  }
  sh[0][threadIdx.x] = (double)s2;
  sh[1][threadIdx.x] = (double)s1;
  sh[2][threadIdx.x] = (double)mx;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      sh[0][threadIdx.x] += sh[0][threadIdx.x + o];
      sh[1][threadIdx.x] += sh[1][threadIdx.x + o];
      sh[2][threadIdx.x] = fmax(sh[2][threadIdx.x], sh[2][threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[blockIdx.x * 3 + 0] = sh[0][0];
    part[blockIdx.x * 3 + 1] = sh[1][0];
    part[blockIdx.x * 3 + 2] = sh[2][0];
  }
}

__global__ void norms_final_kernel(int nblocks, const double *__restrict__ part,
                                   double *__restrict__ out) {
  if (threadIdx.x != 0) return;
  double s2 = 0.0, s1 = 0.0, mx = 0.0;
  for (int b = 0; b < nblocks; b++) {
    s2 += part[b * 3 + 0];
    s1 += part[b * 3 + 1];
    mx = fmax(mx, part[b * 3 + 2]);
  }
  out[0] = sqrt(s2);
  out[1] = s1;
  out[2] = mx;
}

// Partial dots of w with the k columns V[0..k) (column stride ld), kMdCols
// columns per block row (blockIdx.y): a thread reads w once per group of
// columns and keeps one running sum per column, and the block reduces all
// of them with one barrier per halving.  Grid (nblocks, column groups);
// block b's sum for column j goes to part[j * gridDim.x + b].
static constexpr int kMdCols = 8;
static constexpr int kMdBlocks = 2 * kRedBlocks;  // block rows of a column group
template <class T>
__global__ void __launch_bounds__(kRedThreads)
    multidot_tile_kernel(int N, int k, const T *__restrict__ V, int64_t ld,
                         const T *__restrict__ w, double *__restrict__ part) {
  __shared__ double sh[kMdCols][kRedThreads];
  using A = acc_t<T>;
  const int j0 = blockIdx.y * kMdCols;
  const int nc = min(kMdCols, k - j0);
  A s[kMdCols];
#pragma unroll
  for (int c = 0; c < kMdCols; c++) s[c] = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    const A wi = (A)w[i];
#pragma unroll
    for (int c = 0; c < kMdCols; c++)
      if (c < nc) s[c] = fmx((A)V[(int64_t)(j0 + c) * ld + i], wi, s[c]);
  }
#pragma unroll
  for (int c = 0; c < kMdCols; c++) sh[c][threadIdx.x] = (double)s[c];
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
#pragma unroll
      for (int c = 0; c < kMdCols; c++) sh[c][threadIdx.x] += sh[c][threadIdx.x + o];
    }
    __syncthreads();
  }
  if (threadIdx.x < nc) part[(int64_t)(j0 + threadIdx.x) * gridDim.x + blockIdx.x] = sh[threadIdx.x][0];
}

// out[j] = sum over the nblocks partial sums of column j, a warp per column
__global__ void multidot_final_kernel(int k, int nblocks, const double *__restrict__ part,
                                      double *__restrict__ out) {
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (j >= k) return;
  double s = 0.0;
  for (int b = lane; b < nblocks; b += 32) s += part[(int64_t)j * nblocks + b];
  s = warp_sum(s);
  if (lane == 0) out[j] = s;
}

// w -= sum_j h[j] V[:, j]
template <class T>
__global__ void gemv_sub_kernel(int N, int k, const T *__restrict__ V, int64_t ld,
                                const double *__restrict__ h, T *__restrict__ w) {
  using A = acc_t<T>;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    A s = (A)w[i];
#pragma unroll 4
    for (int j = 0; j < k; j++) s = fmx((A)-h[j], (A)V[j * ld + i], s);
    w[i] = (T)s;
  }
}

// y = sum_j c[j] V[:, j]  (c on device)
template <class T>
__global__ void gemv_kernel(int N, int k, const T *__restrict__ V, int64_t ld,
                            const double *__restrict__ c, T *__restrict__ y) {
  using A = acc_t<T>;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    A s = 0;
#pragma unroll 4
    for (int j = 0; j < k; j++) s = fmx((A)c[j], (A)V[j * ld + i], s);
    y[i] = (T)s;
  }
}

template <class T>
__global__ void scale_copy_kernel(int N, const T *x, const double *__restrict__ alpha_inv, T *y) {
  using A = acc_t<T>;
  const A a = (A)(alpha_inv[0] != 0.0 ? 1.0 / alpha_inv[0] : 0.0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    y[i] = (T)((A)x[i] * a);
}

__global__ void axpy_kernel(int N, double a, const double *__restrict__ x, double *__restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    y[i] = fma(a, x[i], y[i]);
}

__global__ void axpy_f32_kernel(int N, double a, const float *__restrict__ x,
                                double *__restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    y[i] = fma(a, (double)x[i], y[i]);
}

// x += t
template <class T>
__global__ void add_kernel(int N, const T *__restrict__ t, T *__restrict__ x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    x[i] = x[i] + t[i];
}

// r = b - r   (r holds A x on entry)
template <class T>
__global__ void sub_from_kernel(int N, const T *__restrict__ b, T *__restrict__ r) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    r[i] = b[i] - r[i];
}

// r = b - r   (r holds A x on entry)
__global__ void residual_kernel(int N, const double *__restrict__ b, double *__restrict__ r) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    r[i] = b[i] - r[i];
}

// y32 = x / s  (normalised down-conversion)
__global__ void to_f32_scaled_kernel(int N, const double *__restrict__ x, double s,
                                     float *__restrict__ y) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    y[i] = (float)(x[i] / s);
}

// y[k] = x[map[k]]
template <class T, class I>
__global__ void gather_kernel(int64_t n, const I *__restrict__ map, const T *__restrict__ x,
                              T *__restrict__ y) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    y[k] = x[map[k]];
}
// y[map[k]] = x[k]
template <class T, class I>
__global__ void scatter_kernel(int64_t n, const I *__restrict__ map, const T *__restrict__ x,
                               T *__restrict__ y) {
  for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    y[map[k]] = x[k];
}

__global__ void to_f32_kernel(int64_t n, const double *__restrict__ x, float *__restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (float)x[i];
}

__global__ void to_f64_kernel(int64_t n, const float *__restrict__ x, double *__restrict__ y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    y[i] = (double)x[i];
}

// ------------------------------------------------------------ SpMV

// y = A x, LPR lanes per row (LPR divides 32)
template <class T, int LPR>
__global__ void spmv_kernel(int N, const int64_t *__restrict__ rowptr,
                            const int *__restrict__ colidx, const T *__restrict__ vals,
                            const T *__restrict__ x, T *__restrict__ y) {
  const int g = (blockIdx.x * blockDim.x + threadIdx.x) / LPR;
  const int l = threadIdx.x % LPR;
  const bool live = g < N;  // the whole warp takes part in the shuffles
  using A = acc_t<T>;
  A s = 0;
  if (live) {
    const int64_t r0 = rowptr[g], r1 = rowptr[g + 1];
    for (int64_t k = r0 + l; k < r1; k += LPR) s = fmx((A)vals[k], (A)__ldg(x + colidx[k]), s);
  }
#pragma unroll
  for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, LPR);
  if (live && l == 0) y[g] = (T)s;
}

// ------------------------------------------------------------ ILU(0)

// first position in [lo, hi) of a sorted column list holding c, or -1
__device__ __forceinline__ int64_t find_col(const int *__restrict__ colidx, int64_t lo, int64_t hi,
                                            int c) {
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (colidx[mid] < c)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// ILU(0) of the rows of one node per CTA, all nodes of one level at once.
//
// The pattern is dense in node blocks (every unknown of a node couples with
// every unknown of every neighbour node; the energy row alone skips pressure
// columns), so the reference's scalar ILU(0) in node-major order is, block
// by block: for each lower neighbour node m (ascending)
//     L_nm   = A_nm U_mm^-1                 (triangular, <= 16 x 16)
//     A_nq  -= L_nm U_mq   for every q > m neighbouring both n and m
// then the dense elimination of the node's own diagonal block and the rest
// of its row.  Fill outside the pattern (energy row x pressure column) is
// dropped, as in ILU(0).  The node's block row lives in shared memory; the
// factored rows of lower nodes are read from global memory (earlier levels).
// A pivot smaller than tau in magnitude (the row-scaled matrix has unit row
// sums) becomes +-tau: in the reference's node-major order an element
// without a pressure datum whose earlier velocity unknowns are all Dirichlet
// rows leaves an exactly singular pressure pivot.
// unknowns per node: nodal fields (<= 3 + 1 + GB_MAX_SPECIES) + P1 pressures
static constexpr int kMaxNodeDofs = 16;

struct IluArgs {
  const int *fu;
  const int64_t *rowptr;
  const int *nbr_ptr, *nbr_node, *nbr_off, *nbr_offT;
  const int *nbr_self;  // every node's own position in its neighbour list
  int dim, nvn, energy;
  int maxnb, lmax, maxnr;
  double tau;
  int *nfix;
};

// Shared memory of one ilu0_block_kernel CTA (element type of size tsize).
static size_t ilu_smem_bytes(size_t tsize, int maxnb, int maxnr, int lmax) {
  return sizeof(int64_t) * (size_t)maxnb * maxnr +                          // srow
         tsize * ((size_t)maxnr * lmax + 3 * kMaxNodeDofs * kMaxNodeDofs + 2 * kMaxNodeDofs) +
         sizeof(int) * (15 * (size_t)maxnb + 4);
}

// ILU(0) of one node's block row (one CTA per node, the nodes of one
// dependency level per launch).  The block row of node n -- its rows over
// the columns of all its neighbours -- lives in shared memory.  For every
// lower neighbour m, in increasing order:
//   step 1  L_nm = A_nm U_mm^-1   (U_mm: m's diagonal block, already final)
//   step 2  A_nq -= L_nm U_mq     for every neighbour q > m of m that is
//                                 also a neighbour of n
// then the diagonal block is factorised in place and the row written back.
// Everything that depends only on the node graph and on finished nodes is
// loaded up front for all m at once (their neighbour-list bounds, own
// positions and row starts).  Per m, "round A" loads m's neighbour list
// (each neighbour's slot in n's list found by binary search in shared
// memory, the shared ones listed through a shared-memory counter), U_mm and
// its reciprocal pivots; it only reads finished nodes, so round A of m+1
// runs during step 2 of m, into the other half of double-buffered tables.
// Step 2 gives each thread one (shared neighbour, column) pair: it loads
// that column of U_mq once and updates every row of n (each target is
// updated once per m, so the list order does not matter).
struct IluRoundA {
  int *tslot, *toff, *toffT, *plist, *np;
};

template <class T>
__device__ __forceinline__ void ilu_round_a(const IluArgs &g, int tid, int nt, int m, int mb,
                                            int mnb, int nm, int Tr, const int64_t *mrow,
                                            int moff, int moffT, const int *snb, int nb,
                                            const T *__restrict__ lu, IluRoundA bufs, T *umm,
                                            T *rdm) {
  for (int t = tid; t < mnb; t += nt) {
    const int q = g.nbr_node[mb + t];
    int slot = -1;
    if (q > m) {
      int lo = 0, hi = nb - 1;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (snb[mid] < q) lo = mid + 1; else hi = mid;
      }
      if (snb[lo] == q) slot = lo;
    }
    bufs.tslot[t] = slot;
    if (slot >= 0) {
      bufs.toff[t] = g.nbr_off[mb + t];
      bufs.toffT[t] = g.nbr_offT[mb + t];
      bufs.plist[atomicAdd(bufs.np, 1)] = t;
    }
  }
  for (int w = tid; w < nm * nm; w += nt) {
    const int dk = w / nm, d2 = w - dk * nm;
    const bool rowkT = dk == Tr;
    T u = (T)0;
    if (d2 >= dk && !(rowkT && d2 >= g.nvn)) u = lu[mrow[dk] + (rowkT ? moffT : moff) + d2];
    umm[dk * kMaxNodeDofs + d2] = u;
    if (d2 == dk) rdm[dk] = (T)1 / u;
  }
}

template <class T>
__global__ void __launch_bounds__(256)
    ilu0_block_kernel(const int *__restrict__ nodes, IluArgs g, const double *__restrict__ A,
                      T *__restrict__ lu) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  int64_t *srow = reinterpret_cast<int64_t *>(sm_raw);          // [maxnb][maxnr] row starts of m
  T *blk = reinterpret_cast<T *>(srow + (size_t)g.maxnb * g.maxnr);  // [maxnr][lmax]
  T *lnm = blk + (size_t)g.maxnr * g.lmax;                       // [16][16] L_nm
  T *umm2 = lnm + kMaxNodeDofs * kMaxNodeDofs;                   // [2][16][16] U_mm
  T *rdm2 = umm2 + 2 * kMaxNodeDofs * kMaxNodeDofs;              // [2][16] 1 / U_mm diagonal
  int *snb = reinterpret_cast<int *>(rdm2 + 2 * kMaxNodeDofs);   // [maxnb] neighbours of n
  int *soff = snb + g.maxnb;                                     // their column offsets
  int *sndof = soff + g.maxnb;                                   // their unknown counts
  int *smb = sndof + g.maxnb;        // lower neighbour m: start of its neighbour list
  int *smnb = smb + g.maxnb;         // its length
  int *smoff = smnb + g.maxnb;       // m's own block in m's rows (offset, energy-row offset)
  int *smoffT = smoff + g.maxnb;
  int *tab = smoffT + g.maxnb;       // [2][4][maxnb] round-A tables, then [2] counters
  int *s_np = tab + 8 * g.maxnb;
  auto bufs = [&](int h) {
    int *b0 = tab + 4 * h * g.maxnb;
    return IluRoundA{b0, b0 + g.maxnb, b0 + 2 * g.maxnb, b0 + 3 * g.maxnb, s_np + h};
  };
  const int n = nodes[blockIdx.x];
  const int tid = threadIdx.x, nt = blockDim.x;
  const int base = g.nbr_ptr[n], nb = g.nbr_ptr[n + 1] - base;
  const int f0 = g.fu[n], nr = g.fu[n + 1] - f0;
  const int Tr = g.energy ? g.dim : -1;  // local index of the energy row
  const int self = g.nbr_self[n];
  if (tid < 2) s_np[tid] = 0;
  for (int s2 = tid; s2 < nb; s2 += nt) {
    const int q = g.nbr_node[base + s2];
    snb[s2] = q;
    soff[s2] = g.nbr_off[base + s2];
    const int fq = g.fu[q];
    sndof[s2] = g.fu[q + 1] - fq;
    if (s2 < self) {
      const int mb = g.nbr_ptr[q];
      const int ms = g.nbr_self[q];
      smb[s2] = mb;
      smnb[s2] = g.nbr_ptr[q + 1] - mb;
      smoff[s2] = g.nbr_off[mb + ms];
      smoffT[s2] = g.nbr_offT[mb + ms];
      for (int dk = 0; dk < g.fu[q + 1] - fq; dk++)
        srow[(size_t)s2 * g.maxnr + dk] = g.rowptr[fq + dk];
    }
  }
  __syncthreads();
  const int L = soff[nb - 1] + sndof[nb - 1];
  // load the block row (full layout; energy-row pressure columns held at 0)
  for (int c = tid; c < L; c += nt) {
    int lo = 0, hi = nb - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (soff[mid] <= c) lo = mid; else hi = mid - 1;
    }
    const int d = c - soff[lo];
    for (int r = 0; r < nr; r++) {
      if (r == Tr) {
        blk[r * g.lmax + c] = d >= g.nvn ? (T)0 : (T)A[g.rowptr[f0 + r] + g.nbr_offT[base + lo] + d];
      } else {
        blk[r * g.lmax + c] = (T)A[g.rowptr[f0 + r] + c];
      }
    }
  }
  if (self > 0)
    ilu_round_a<T>(g, tid, nt, snb[0], smb[0], smnb[0], sndof[0], Tr, srow, smoff[0], smoffT[0],
                   snb, nb, lu, bufs(0), umm2, rdm2);
  __syncthreads();
  for (int sm = 0; sm < self; sm++) {
    const int h = sm & 1;
    const IluRoundA cur = bufs(h);
    const T *umm = umm2 + h * kMaxNodeDofs * kMaxNodeDofs;
    const T *rdm = rdm2 + h * kMaxNodeDofs;
    const int nm = sndof[sm], cm = soff[sm];
    const int64_t *mrow = srow + (size_t)sm * g.maxnr;
    // step 1: L_nm = A_nm U_mm^-1, a warp per row (lane d holds the row's
    // entry in m's column d): per pivot one shuffle, then every later
    // column updated at once
    for (int r = tid >> 5; r < nr; r += nt >> 5) {
      const int lane = tid & 31;
      T *br = blk + (size_t)r * g.lmax + cm;
      T v = lane < nm ? br[lane] : (T)0;
      for (int dk = 0; dk < nm; dk++) {
        if (r == Tr && dk >= g.nvn) {  // energy row: no pressure columns
          if (lane == 0) lnm[r * kMaxNodeDofs + dk] = (T)0;
          continue;
        }
        const T l = __shfl_sync(0xffffffffu, v, dk) * rdm[dk];
        if (lane == dk) v = l;
        if (lane == 0) lnm[r * kMaxNodeDofs + dk] = l;
        if (lane > dk && lane < nm && !(r == Tr && lane >= g.nvn))
          v -= l * umm[dk * kMaxNodeDofs + lane];  // zero where U_mm has no entry
      }
      if (lane < nm) br[lane] = v;
    }
    __syncthreads();
    // round A of the next neighbour, into the other half of the tables
    // (its counter was reset before the barrier that ended its last use)
    if (sm + 1 < self)
      ilu_round_a<T>(g, tid, nt, snb[sm + 1], smb[sm + 1], smnb[sm + 1], sndof[sm + 1], Tr,
                     srow + (size_t)(sm + 1) * g.maxnr, smoff[sm + 1], smoffT[sm + 1], snb, nb,
                     lu, bufs(h ^ 1), umm2 + (h ^ 1) * kMaxNodeDofs * kMaxNodeDofs,
                     rdm2 + (h ^ 1) * kMaxNodeDofs);
    // step 2: A_nq -= L_nm U_mq, one thread per (shared neighbour, column d)
    // loading the column of U_mq once and updating every row of n
    const int np = *cur.np;
    for (int f = tid; f < np * g.maxnr; f += nt) {
      const int k = f / g.maxnr, d = f - k * g.maxnr;
      const int t = cur.plist[k], slot = cur.tslot[t];
      if (d >= sndof[slot]) continue;
      const int off = cur.toff[t], offT = cur.toffT[t];
      T u[kMaxNodeDofs];
#pragma unroll
      for (int dk = 0; dk < kMaxNodeDofs; dk++) {
        u[dk] = (T)0;
        if (dk < nm && !(dk == Tr && d >= g.nvn)) u[dk] = lu[mrow[dk] + (dk == Tr ? offT : off) + d];
      }
      T *col = blk + soff[slot] + d;
      for (int r = 0; r < nr; r++) {
        if (r == Tr && d >= g.nvn) continue;
        T acc = (T)0;
#pragma unroll
        for (int dk = 0; dk < kMaxNodeDofs; dk++) {
          if (dk >= nm) break;
          if (dk == Tr && d >= g.nvn) continue;
          acc += lnm[r * kMaxNodeDofs + dk] * u[dk];
        }
        col[(size_t)r * g.lmax] -= acc;
      }
    }
    __syncthreads();
    if (tid == 0) *cur.np = 0;  // free for the round A of neighbour sm + 2
  }
  // own diagonal block and the rest of the row
  const int cs = soff[self];
  for (int dk = 0; dk < nr; dk++) {
    if (tid == 0) {
      const T p = blk[dk * g.lmax + cs + dk];
      if (fabs((double)p) < g.tau) {
        blk[dk * g.lmax + cs + dk] = p < (T)0 ? (T)-g.tau : (T)g.tau;
        atomicAdd(g.nfix, 1);
      }
    }
    __syncthreads();
    const T piv = blk[dk * g.lmax + cs + dk];
    const int c0 = cs + dk + 1;
    for (int r = dk + 1; r < nr; r++) {
      if (r == Tr && dk >= g.nvn) continue;
      const T l = blk[r * g.lmax + cs + dk] / piv;
      for (int c = c0 + tid; c < L; c += nt) {
        const T u = blk[dk * g.lmax + c];
        if (u == (T)0) continue;
        if (r == Tr) {
          // energy row: pressure columns are outside the pattern
          int lo = 0, hi = nb - 1;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (soff[mid] <= c) lo = mid; else hi = mid - 1;
          }
          if (c - soff[lo] >= g.nvn) continue;
        }
        blk[r * g.lmax + c] -= l * u;
      }
    }
    __syncthreads();
    if (tid < nr && tid > dk && !(tid == Tr && dk >= g.nvn))
      blk[tid * g.lmax + cs + dk] = blk[tid * g.lmax + cs + dk] / piv;
    __syncthreads();
  }
  // write back
  for (int c = tid; c < L; c += nt) {
    int lo = 0, hi = nb - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (soff[mid] <= c) lo = mid; else hi = mid - 1;
    }
    const int d = c - soff[lo];
    for (int r = 0; r < nr; r++) {
      if (r == Tr) {
        if (d < g.nvn) lu[g.rowptr[f0 + r] + g.nbr_offT[base + lo] + d] = blk[r * g.lmax + c];
      } else {
        lu[g.rowptr[f0 + r] + c] = blk[r * g.lmax + c];
      }
    }
  }
}

// Sync-free triangular solves: one launch per sweep, one CTA per node at a
// time.  The nodes are numbered ("tickets") in the order of their
// dependency levels (the level schedule of the sweep: all of level 0, then
// level 1, ...; independent problems in one matrix interleave), and CTA b of
// a G-CTA grid takes tickets b, b + G, b + 2G, ... in turn -- no atomic, and
// a CTA reads its next node's ticket entry while it works on the current
// one.  Per ticket a table holds the node's first unknown, unknown count and
// block-inverse offset; per row one holds its off-node segment; the factor
// values and column indices of the segments are stored in the sweep's own
// (level-sorted) order, so a CTA reaches its rows' data in two dependent
// loads.  A sweep
// reads its right-hand side from one vector and writes its solution into
// another that was filled beforehand with an "unpublished" sentinel (a
// signalling NaN: arithmetic never produces one, so every computed value,
// NaNs included, differs from it).  A node needs exactly the solution
// values its rows reference, so it polls those values themselves until none
// is the sentinel -- no per-node flag, no fence: each value is published by
// one single-copy-atomic store.  The node is solved in two stages:
//   A  all warps: for every row of the node, the right-hand side less the
//      dot product with the solution values of OTHER nodes (the long part of
//      the row, rows spread over the warps; each lane keeps its polled values
//      in registers and adds them in a fixed order, so the result does not
//      depend on arrival order);
//   B  warp 0, lane r for row r: row r of the node's precomputed diagonal-
//      block inverse (block_inverse_kernel, in shared memory) times those
//      values -- independent products, no chain of substitution steps.
// A warp loads its first row's factor values and column indices, and the
// CTA the block inverse, before it polls, so only the gather of the
// solution values stays on the critical path.  A node depends
// only on nodes of lower levels, which hold earlier tickets; every CTA of the
// grid is resident and takes its tickets in increasing order, so the lowest
// unfinished ticket always has all its dependencies published and is held
// by a CTA that is working on it: the sweep makes progress.  Every wait is bounded: past spin_limit polls the
// CTA records an error, computes and publishes anyway (so no other CTA can
// wait forever), every later wait of the sweep stops within 1024 polls, and
// the host reports the failure after the sweep.  A legitimate wait lasts
// microseconds; the default limit (kSpinLimit) is ~0.3 s.
//
// Row structure used by the split: a node's unknowns are contiguous and
// every row of the node holds every own-node column except the energy row,
// which lacks the pressure columns (they come last).  So in row i (local
// index r) the own-node columns below the diagonal are the r entries just
// before it, and those above are the next nr-1-r entries (nvn-1-r for the
// energy row).
static constexpr long long kSpinLimit = 1LL << 22;
// row entries per lane loaded before the wait: 320 a row in FP32, 256 in
// FP64 (where ten would spill at the 64 registers of four CTAs per SM)
template <class T> constexpr int kPrefetchOf = sizeof(T) == 4 ? 10 : 8;
static constexpr int kTrsvThreads = 256;

struct TrsvArgs {
  // the sync-free sweep's own tables, set per sweep: per ticket the node's
  // (unknown count << 32 | first unknown) and the offset of its block
  // inverse; per unknown the row's off-node segment [begin, end); the
  // segments' column indices in sweep (level-sorted) order
  const longlong2 *tick;
  const longlong2 *seg;
  const int *cols;
  const int *fu;
  const int64_t *rowptr;
  const int *colidx;
  const int64_t *diag;
  const int64_t *inv_ptr;  // node n's diagonal-block inverses start at inv_ptr[n] (L's, then U's)
  int num_nodes;
  int Tr;              // local index of the energy row, -1 without energy
  int nvn;             // nodal fields per node
  int *error;          // set when a wait gave up
  long long spin_limit;  // polls before a wait gives up
};

// the "unpublished" sentinels: signalling NaNs (exponent all ones, quiet bit
// clear, non-zero payload)
static constexpr unsigned long long kUnpub64 = 0xFFF5DEAD5EEDF00DULL;
static constexpr unsigned kUnpub32 = 0xFFA5EED5u;
__device__ __forceinline__ bool unpublished(double v) {
  return (unsigned long long)__double_as_longlong(v) == kUnpub64;
}
__device__ __forceinline__ bool unpublished(float v) { return __float_as_uint(v) == kUnpub32; }
__device__ __forceinline__ void set_unpublished(double *p) {
  *p = __longlong_as_double((long long)kUnpub64);
}
__device__ __forceinline__ void set_unpublished(float *p) { *p = __uint_as_float(kUnpub32); }

__device__ __forceinline__ double ld_relaxed(const double *p) {
  double v;
  asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ float ld_relaxed(const float *p) {
  float v;
  asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(double *p, double v) {
  asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(float *p, float v) {
  asm volatile("st.relaxed.gpu.global.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}

// fill a sweep's output with the sentinel
template <class T>
__global__ void trsv_prepare_kernel(int64_t n, T *x) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    set_unpublished(x + i);
}

// one solution value, polled until published (bounded; 0 once given up)
template <class T>
__device__ __forceinline__ T poll_value(const T *p, bool &gave_up, const int *error,
                                        long long spin_limit) {
  T v = ld_relaxed(p);
  long long polls = 0;
  while (unpublished(v)) {
    if (gave_up || ++polls > spin_limit || ((polls & 1023) == 0 && *(volatile const int *)error)) {
      gave_up = true;
      return (T)0;
    }
    v = ld_relaxed(p);
  }
  return v;
}

// Dense inverses of every node's diagonal blocks of the factors: of the
// unit lower block of L and of the upper block of U (nr x nr each, stored
// column by column, entry (r, c) at c * nr + r; L's first).  With them a
// sweep finishes a node with one small matrix-vector product,
// x_n = D^-1 (b_n - off-node part), whose products are independent, in place
// of a substitution whose steps each wait for the previous one.  Block
// layout: a node's unknowns are contiguous and every row of the node holds
// every own-node column except the energy row, which lacks the pressure
// columns (they come last); row r's own-node columns start r entries before
// its diagonal.  One warp per node, lane j computes column j of both
// inverses by substitution.
template <class T>
__global__ void block_inverse_kernel(TrsvArgs g, const T *__restrict__ lu, T *__restrict__ inv) {
  using A = acc_t<T>;
  const int wpb = blockDim.x >> 5, j = threadIdx.x & 31;
  for (int n = blockIdx.x * wpb + (threadIdx.x >> 5); n < g.num_nodes; n += gridDim.x * wpb) {
    const int f0 = g.fu[n], nr = g.fu[n + 1] - f0;
    T *Li = inv + g.inv_ptr[n], *Ui = Li + nr * nr;
    if (j >= nr) continue;
    A x[kMaxNodeDofs];
    // column j of L^-1: x_i = [i == j] - sum_{j <= c < i} L(i, c) x_c
    for (int i = 0; i < nr; i++) {
      A v = i == j ? (A)1 : (A)0;
      if (i > j) {
        const int64_t rb = g.diag[f0 + i] - i;  // row i's own-node columns start here
        for (int c = j; c < i; c++) v -= (A)lu[rb + c] * x[c];
      }
      x[i] = v;
      Li[(size_t)j * nr + i] = (T)v;
    }
    // column j of U^-1: x_i = ([i == j] - sum_{i < c <= j} U(i, c) x_c) / U(i, i)
    for (int i = nr - 1; i >= 0; i--) {
      A v = (A)0;
      if (i <= j) {
        const int64_t di = g.diag[f0 + i];
        const int cend = i == g.Tr ? min(j, g.nvn - 1) : j;  // energy row: no pressure columns
        v = i == j ? (A)1 : (A)0;
        for (int c = i + 1; c <= cend; c++) v -= (A)lu[di + (c - i)] * x[c];
        v = v / (A)lu[di];
      }
      x[i] = v;
      Ui[(size_t)j * nr + i] = (T)v;
    }
  }
}

// Stage B, shared by the sweeps: lane r of the calling warp returns row r of
// D^-1 bv, D^-1 the node's block inverse (entry (r, c) at inv_s[c * 16 + r],
// lower triangular for L, upper for U), bv the rows' right-hand sides less
// their off-node parts; the products are added in column order.
template <class A, bool LOWER>
__device__ __forceinline__ A node_block_apply(int lane, int nr, const A *inv_s, const A *bv) {
  A v = (A)0;
  if (lane < nr) {
    for (int c = 0; c < nr; c++)
      if (LOWER ? c <= lane : c >= lane) v = fmx(inv_s[c * kMaxNodeDofs + lane], bv[c], v);
  }
  return v;
}

// Copies every row's off-node segments of src into dst in the sweeps'
// level-sorted order (entry p of a segment from segment start + rel[p]), so
// the sync-free sweeps read factor values and column indices contiguously,
// without the extra indirection.  One warp per row.
template <class E>
__global__ void sweep_gather_kernel(int N, const longlong2 *__restrict__ segL,
                                    const longlong2 *__restrict__ segU,
                                    const uint16_t *__restrict__ rel, const E *__restrict__ src,
                                    E *__restrict__ dst) {
  const int wpb = blockDim.x >> 5, lane = threadIdx.x & 31;
  for (int i = blockIdx.x * wpb + (threadIdx.x >> 5); i < N; i += gridDim.x * wpb) {
    for (int h = 0; h < 2; h++) {
      const longlong2 sg = h ? segU[i] : segL[i];
      for (int64_t p = sg.x + lane; p < sg.y; p += 32) dst[p] = src[sg.x + rel[p]];
    }
  }
}

template <class T, bool LOWER>
__global__ void __launch_bounds__(kTrsvThreads, 4)
    trsv_sync_free_kernel(TrsvArgs g, const T *__restrict__ lus, const T *__restrict__ binv,
                          const T *__restrict__ b, T *x) {
  using A = acc_t<T>;
  constexpr int kPf = kPrefetchOf<T>;
  __shared__ A bv[kMaxNodeDofs];                      // per row: rhs less the off-node part
  __shared__ A inv_s[kMaxNodeDofs * kMaxNodeDofs];    // the node's block inverse, by column
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NW = kTrsvThreads / 32;
  const unsigned nt = (unsigned)g.num_nodes, stride = gridDim.x;
  unsigned t = blockIdx.x;
  longlong2 tk = t < nt ? g.tick[t] : make_longlong2(0, 0);
  for (; t < nt; t += stride) {
    const int f0 = (int)(tk.x & 0xffffffffll), nr = (int)(tk.x >> 32);
    const int64_t inv_off = tk.y;
    // before polling: everything that does not depend on the sweep
    A pv[kPf];
    int pc[kPf];
    int64_t pr0 = 0, pr1 = 0;
    if (warp < nr) {
      const longlong2 sg = g.seg[f0 + warp];
      pr0 = sg.x;
      pr1 = sg.y;
#pragma unroll
      for (int k = 0; k < kPf; k++) {
        const int64_t p = pr0 + lane + 32 * k;
        pv[k] = p < pr1 ? (A)lus[p] : (A)0;
        pc[k] = p < pr1 ? g.cols[p] : -1;
      }
    }
    for (int w = tid; w < nr * nr; w += kTrsvThreads) {
      const int c = w / nr;
      inv_s[c * kMaxNodeDofs + (w - c * nr)] = (A)binv[inv_off + w];
    }
    // this CTA's next node (static round-robin tickets)
    if (t + stride < nt) tk = g.tick[t + stride];
    // stage A
    bool gave_up = false;
    for (int r = warp; r < nr; r += NW) {
      const A rhs_r = (A)__ldcg(b + f0 + r);
      A s0 = 0;
      int64_t p, p1;
      if (r == warp) {
        // the prefetched row: load all its values at once, then add them in
        // the fixed (level-sorted, oldest first) order, each as soon as it
        // and every earlier one are published -- the values published long
        // ago are added while the newest ones are still awaited; a wait
        // re-polls only the value it waits for, so waiting warps issue few
        // instructions
        A zv[kPf];
        unsigned pending = 0;
#pragma unroll
        for (int k = 0; k < kPf; k++) {
          zv[k] = 0;
          if (pc[k] >= 0) {
            const T v = ld_relaxed(x + pc[k]);
            if (unpublished(v)) pending |= 1u << k; else zv[k] = (A)v;
          }
        }
        long long polls = 0;
#pragma unroll
        for (int k = 0; k < kPf; k++) {
          while (!gave_up && (pending & (1u << k))) {
            if (++polls > g.spin_limit ||
                ((polls & 1023) == 0 && *(volatile const int *)g.error)) {
              gave_up = true;
              break;
            }
            const T v = ld_relaxed(x + pc[k]);
            if (!unpublished(v)) {
              zv[k] = (A)v;
              pending &= ~(1u << k);
            }
          }
          if (pc[k] >= 0) s0 = fmx(pv[k], zv[k], s0);
        }
        p = pr0 + lane + 32 * kPf;
        p1 = pr1;
      } else {
        const longlong2 sg = g.seg[f0 + r];
        p = sg.x + lane;
        p1 = sg.y;
      }
      for (; p < p1; p += 32)
        s0 = fmx((A)lus[p], (A)poll_value(x + g.cols[p], gave_up, g.error, g.spin_limit), s0);
      const A sum = wsum(s0);
      if (lane == 0) bv[r] = rhs_r - sum;
    }
    if (__syncthreads_or(gave_up) && tid == 0) atomicExch(g.error, 1);
    // stage B
    if (warp == 0) {
      const A v = node_block_apply<A, LOWER>(lane, nr, inv_s, bv);
      if (lane < nr) st_relaxed(x + f0 + lane, (T)v);
    }
    __syncthreads();
  }
}

// The same sweep with one warp per node, for meshes whose nodes have few
// unknowns and short rows (QUAD9 problems: 2-6 rows of at most a few dozen
// off-node entries).  A node's rows go to lane groups of G = 32 / R lanes
// (R: the row count rounded up to a power of two), a group sums its row in
// a fixed order (lane by lane, then a butterfly within the group), and the
// block inverse is applied with one shuffle per row -- no shared memory and
// no barrier, so a warp needs far fewer resources than a CTA and many more
// nodes are in flight (each 128-thread CTA holds four).  Warp w of the grid
// takes tickets w, w + W, ... (W warps in all), with the same progress
// argument as the CTA sweep.  Used when every node has at most kWarpMaxRows
// rows and every row's off-node segment fits its group's prefetch window:
// always in FP32, in FP64 only for wide levels (Solver::init).
static constexpr int kWarpMaxRows = 8;
static constexpr int kPrefetchW = 8;
static constexpr int kWarpSweepThreads = 128;

template <class T, bool LOWER>
__global__ void __launch_bounds__(kWarpSweepThreads)
    trsv_sync_free_warp_kernel(TrsvArgs g, const T *__restrict__ lus,
                               const T *__restrict__ binv, const T *__restrict__ b, T *x) {
  using A = acc_t<T>;
  const int lane = threadIdx.x & 31;
  const unsigned nt = (unsigned)g.num_nodes;
  const unsigned wpb = blockDim.x >> 5, stride = gridDim.x * wpb;
  unsigned t = blockIdx.x * wpb + (threadIdx.x >> 5);
  longlong2 tk = t < nt ? g.tick[t] : make_longlong2(0, 0);
  for (; t < nt; t += stride) {
    const int f0 = (int)(tk.x & 0xffffffffll), nr = (int)(tk.x >> 32);
    const int64_t inv_off = tk.y;
    int R = 1;
    while (R < nr) R <<= 1;
    const int G = 32 / R;                     // lanes per row
    const int r = lane / G, gl = lane - r * G;
    const bool act = r < nr;
    A pv[kPrefetchW];
    int pc[kPrefetchW];
    int64_t pr0 = 0, pr1 = 0;
    if (act) {
      const longlong2 sg = g.seg[f0 + r];
      pr0 = sg.x;
      pr1 = sg.y;
    }
#pragma unroll
    for (int k = 0; k < kPrefetchW; k++) {
      const int64_t p = pr0 + gl + (int64_t)G * k;
      pv[k] = p < pr1 ? (A)lus[p] : (A)0;
      pc[k] = p < pr1 ? g.cols[p] : -1;
    }
    // lane c < nr holds row c of the block inverse
    A dv[kWarpMaxRows];
#pragma unroll
    for (int c = 0; c < kWarpMaxRows; c++)
      dv[c] = (lane < nr && c < nr) ? (A)binv[inv_off + (int64_t)c * nr + lane] : (A)0;
    const A rhs_r = act ? (A)__ldcg(b + f0 + r) : (A)0;
    if (t + stride < nt) tk = g.tick[t + stride];
    // stage A: the row's off-node sum, values added in the fixed order as
    // they arrive (a wait re-polls only its own value)
    bool gave_up = false;
    A zv[kPrefetchW];
    unsigned pending = 0;
#pragma unroll
    for (int k = 0; k < kPrefetchW; k++) {
      zv[k] = 0;
      if (pc[k] >= 0) {
        const T v = ld_relaxed(x + pc[k]);
        if (unpublished(v)) pending |= 1u << k; else zv[k] = (A)v;
      }
    }
    A s0 = 0;
    long long polls = 0;
#pragma unroll
    for (int k = 0; k < kPrefetchW; k++) {
      while (!gave_up && (pending & (1u << k))) {
        if (++polls > g.spin_limit || ((polls & 1023) == 0 && *(volatile const int *)g.error)) {
          gave_up = true;
          break;
        }
        const T v = ld_relaxed(x + pc[k]);
        if (!unpublished(v)) {
          zv[k] = (A)v;
          pending &= ~(1u << k);
        }
      }
      if (pc[k] >= 0) s0 = fmx(pv[k], zv[k], s0);
    }
    for (int64_t p = pr0 + gl + (int64_t)G * kPrefetchW; p < pr1; p += G)
      s0 = fmx((A)lus[p], (A)poll_value(x + g.cols[p], gave_up, g.error, g.spin_limit), s0);
    for (int o = G >> 1; o > 0; o >>= 1) s0 += __shfl_xor_sync(0xffffffffu, s0, o);
    const A bvr = rhs_r - s0;
    // stage B: x_n = D^-1 (rhs - off-node part), products in column order
    A v = 0;
#pragma unroll
    for (int c = 0; c < kWarpMaxRows; c++) {
      if (c < nr) {
        const A bc = __shfl_sync(0xffffffffu, bvr, c * G);
        if (lane < nr && (LOWER ? c <= lane : c >= lane)) v = fmx(dv[c], bc, v);
      }
    }
    if (lane < nr) st_relaxed(x + f0 + lane, (T)v);
    if (__any_sync(0xffffffffu, gave_up) && lane == 0) atomicExch(g.error, 1);
  }
}

// One dependency level of a triangular sweep, one CTA per node: the nodes of
// a level do not depend on each other, so the launch boundary is the only
// synchronisation.  Same two stages as the sync-free sweep (rows over the
// warps, then the in-node solve over the lanes of warp 0), in place on z;
// used for short level schedules (the multicoloured order), launched level
// after level from a captured graph.
template <class T, bool LOWER>
__global__ void __launch_bounds__(kTrsvThreads)
    trsv_level_cta_kernel(const int *__restrict__ nodes, TrsvArgs g, const T *__restrict__ lu,
                          const T *__restrict__ binv, T *__restrict__ z) {
  using A = acc_t<T>;
  __shared__ A bv[kMaxNodeDofs];
  __shared__ A inv_s[kMaxNodeDofs * kMaxNodeDofs];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  constexpr int NW = kTrsvThreads / 32;
  const int n = nodes[blockIdx.x];
  const int f0 = g.fu[n], nr = g.fu[n + 1] - f0;
  {
    const T *bi = binv + g.inv_ptr[n] + (LOWER ? 0 : nr * nr);
    for (int w = tid; w < nr * nr; w += kTrsvThreads) {
      const int c = w / nr;
      inv_s[c * kMaxNodeDofs + (w - c * nr)] = (A)bi[w];
    }
  }
  // rows over the warps; a node's own right-hand side is read before any
  // of its values is written (only this CTA writes them, after the barrier)
  for (int r = warp; r < nr; r += NW) {
    const int i = f0 + r;
    const int64_t di = g.diag[i];
    const int na = (r == g.Tr ? g.nvn : nr) - 1 - r;
    const int64_t p0 = LOWER ? g.rowptr[i] : di + 1 + na;
    const int64_t p1 = LOWER ? di - r : g.rowptr[i + 1];
    const A rhs_r = (A)z[i];
    A s0 = 0, s1 = 0;
    int64_t p = p0 + lane;
    for (; p + 32 < p1; p += 64) {
      s0 = fmx((A)lu[p], (A)z[g.colidx[p]], s0);
      s1 = fmx((A)lu[p + 32], (A)z[g.colidx[p + 32]], s1);
    }
    if (p < p1) s0 = fmx((A)lu[p], (A)z[g.colidx[p]], s0);
    const A sum = wsum(s0 + s1);
    if (lane == 0) bv[r] = rhs_r - sum;
  }
  __syncthreads();
  if (warp == 0) {
    const A v = node_block_apply<A, LOWER>(lane, nr, inv_s, bv);
    if (lane < nr) z[f0 + lane] = (T)v;
  }
}

// the sweeps' view of the preconditioner layout (the sync-free sweep sets
// its tickets, segments and columns)
static TrsvArgs trsv_args(const Solver *S) {
  TrsvArgs g;
  g.tick = nullptr;
  g.seg = nullptr;
  g.cols = nullptr;
  g.fu = S->P.fu;
  g.rowptr = S->P.rowptr;
  g.colidx = S->P.colidx;
  g.diag = S->P.diag;
  g.inv_ptr = S->d_inv_ptr;
  g.num_nodes = S->C->L.num_nodes;
  g.Tr = S->C->L.energy ? S->C->L.dim : -1;
  g.nvn = S->C->L.nvn;
  g.error = nullptr;
  g.spin_limit = S->C->sweep_spin_limit > 0 ? S->C->sweep_spin_limit : kSpinLimit;
  return g;
}

// ------------------------------------------------------------ schedule

void build_ilu_schedule(const Layout &L, IluSchedule &S) {
  const int nn = L.num_nodes;
  std::vector<int> lev(nn, 0);
  int maxl = 0;
  for (int n = 0; n < nn; n++) {
    int l = 0;
    for (int q = L.nbr_ptr[n]; q < L.nbr_ptr[n + 1]; q++) {
      const int m = L.nbr_node[q];
      if (m < n) l = std::max(l, lev[m] + 1);
    }
    lev[n] = l;
    maxl = std::max(maxl, l);
  }
  S.lo_ptr.assign(maxl + 2, 0);
  for (int n = 0; n < nn; n++) S.lo_ptr[lev[n] + 1]++;
  for (int l = 0; l <= maxl; l++) S.lo_ptr[l + 1] += S.lo_ptr[l];
  S.lo_nodes.resize(nn);
  {
    std::vector<int> fill(maxl + 1, 0);
    for (int n = 0; n < nn; n++) S.lo_nodes[S.lo_ptr[lev[n]] + fill[lev[n]]++] = n;
  }
  S.lev = lev;
  std::vector<int> levu(nn, 0);
  int maxu = 0;
  for (int n = nn - 1; n >= 0; n--) {
    int l = 0;
    for (int q = L.nbr_ptr[n]; q < L.nbr_ptr[n + 1]; q++) {
      const int m = L.nbr_node[q];
      if (m > n) l = std::max(l, levu[m] + 1);
    }
    levu[n] = l;
    maxu = std::max(maxu, l);
  }
  S.up_ptr.assign(maxu + 2, 0);
  for (int n = 0; n < nn; n++) S.up_ptr[levu[n] + 1]++;
  for (int l = 0; l <= maxu; l++) S.up_ptr[l + 1] += S.up_ptr[l];
  S.up_nodes.resize(nn);
  {
    std::vector<int> fill(maxu + 1, 0);
    for (int n = 0; n < nn; n++) S.up_nodes[S.up_ptr[levu[n]] + fill[levu[n]]++] = n;
  }
  S.levu = levu;
}

// ------------------------------------------------------------ Solver

Solver::~Solver() {
  if (prec64) cudaGraphExecDestroy(prec64);
  if (prec32) cudaGraphExecDestroy(prec32);
  void *p[] = {d_lu, d_lu32, d_lus, d_lus32, d_binv, d_binv32, d_Z, d_a32, d_diag, d_lo_nodes, d_up_nodes, d_scale, d_work, d_flags,
               d_sweep_y, d_V, d_V32, d_t, d_w, d_r, d_xs, d_t32, d_w32};
  for (void *q : p)
    if (q) cudaFree(q);
  for (void *q : owned)
    if (q) cudaFree(q);
  if (h_work) cudaFreeHost(h_work);
  if (h_segout) cudaFreeHost(h_segout);
}

#define GB_CU(call, what)                          \
  do {                                             \
    cudaError_t e_ = (call);                       \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

int Solver::init(Context *c, int krylov) {
  C = c;
  N = c->L.N;
  nnz = c->L.nnz;
  max_krylov = krylov;
  const Layout &L = c->L;
  std::vector<int64_t> diag(N);
  for (int i = 0; i < N; i++) {
    auto b = L.colidx.begin() + L.rowptr[i], e = L.colidx.begin() + L.rowptr[i + 1];
    auto it = std::lower_bound(b, e, i);
    diag[i] = (int64_t)(it - L.colidx.begin());
  }
  GB_CU(cudaMalloc(&d_diag, sizeof(int64_t) * N), "diag");
  GB_CU(cudaMemcpy(d_diag, diag.data(), sizeof(int64_t) * N, cudaMemcpyHostToDevice), "diag");
  ordering = c->ilu_ordering;
  Layout Lp;
  const Layout *LP = &L;  // the layout the factors live in
  if (ordering == 1) {
    std::vector<int> perm, um;
    std::vector<int64_t> vm;
    multicolour_order(L, perm);
    permute_layout(L, perm, Lp, um, vm);
    std::vector<int64_t> pdiag(N);
    for (int i = 0; i < N; i++) {
      auto b = Lp.colidx.begin() + Lp.rowptr[i], e = Lp.colidx.begin() + Lp.rowptr[i + 1];
      pdiag[i] = (int64_t)(std::lower_bound(b, e, i) - Lp.colidx.begin());
    }
    auto up = [&](auto &vec, const char *what) -> void * {
      void *d = nullptr;
      if (cudaMalloc(&d, sizeof(vec[0]) * vec.size()) != cudaSuccess) return nullptr;
      owned.push_back(d);
      if (cudaMemcpy(d, vec.data(), sizeof(vec[0]) * vec.size(), cudaMemcpyHostToDevice) !=
          cudaSuccess)
        return nullptr;
      (void)what;
      return d;
    };
    P.fu = (const int *)up(Lp.fu, "fu");
    P.rowptr = (const int64_t *)up(Lp.rowptr, "rowptr");
    P.colidx = (const int *)up(Lp.colidx, "colidx");
    P.diag = (const int64_t *)up(pdiag, "diag");
    P.nbr_ptr = (const int *)up(Lp.nbr_ptr, "nbr");
    P.nbr_node = (const int *)up(Lp.nbr_node, "nbr");
    P.nbr_off = (const int *)up(Lp.nbr_off, "nbr");
    P.nbr_offT = (const int *)up(Lp.nbr_offT, "nbr");
    d_umap = (int *)up(um, "umap");
    d_vmap = (int64_t *)up(vm, "vmap");
    if (!P.fu || !P.rowptr || !P.colidx || !P.diag || !P.nbr_ptr || !P.nbr_node || !P.nbr_off ||
        !P.nbr_offT || !d_umap || !d_vmap)
      return fail("multicoloured ILU(0) layout: device allocation");
    GB_CU(cudaMalloc(&d_Ap, sizeof(double) * nnz), "permuted matrix");
    owned.push_back(d_Ap);
    GB_CU(cudaMalloc(&d_tp, sizeof(double) * N), "permuted vector");
    owned.push_back(d_tp);
    LP = &Lp;
  } else {
    P.fu = c->d_fu;
    P.rowptr = c->d_rowptr;
    P.colidx = c->d_colidx;
    P.diag = d_diag;
    P.nbr_ptr = c->d_nbr_ptr;
    P.nbr_node = c->d_nbr_node;
    P.nbr_off = c->d_nbr_off;
    P.nbr_offT = c->d_nbr_offT;
  }
  std::vector<int64_t> ip(LP->num_nodes + 1, 0);  // block-inverse offsets
  {
    std::vector<int> self(LP->num_nodes);
    for (int n = 0; n < LP->num_nodes; n++) {
      auto b = LP->nbr_node.begin() + LP->nbr_ptr[n], e = LP->nbr_node.begin() + LP->nbr_ptr[n + 1];
      self[n] = (int)(std::lower_bound(b, e, n) - b);
    }
    int *d = nullptr;
    GB_CU(cudaMalloc(&d, sizeof(int) * self.size()), "neighbour self positions");
    owned.push_back(d);
    GB_CU(cudaMemcpy(d, self.data(), sizeof(int) * self.size(), cudaMemcpyHostToDevice),
          "neighbour self positions");
    P.nbr_self = d;
    // offsets of every node's diagonal-block inverses (L's and U's, nr^2 each)
    for (int n = 0; n < LP->num_nodes; n++) {
      const int64_t nr = LP->fu[n + 1] - LP->fu[n];
      ip[n + 1] = ip[n] + 2 * nr * nr;
    }
    inv_len = ip.back();
    GB_CU(cudaMalloc(&d_inv_ptr, sizeof(int64_t) * ip.size()), "block inverse offsets");
    owned.push_back(d_inv_ptr);
    GB_CU(cudaMemcpy(d_inv_ptr, ip.data(), sizeof(int64_t) * ip.size(), cudaMemcpyHostToDevice),
          "block inverse offsets");
    GB_CU(cudaMalloc(&d_binv, sizeof(double) * inv_len), "block inverses");
  }
  IluSchedule S;
  build_ilu_schedule(*LP, S);
  lo_ptr = S.lo_ptr;
  up_ptr = S.up_ptr;
  num_levels = (int)lo_ptr.size() - 1;
  {
    std::vector<uint16_t> rel;
    if (build_sweep_order(*LP, S.lev, S.levu, rel)) return fail("a matrix row is too long for the sweeps");
    GB_CU(cudaMalloc(&d_sweep_rel, sizeof(uint16_t) * rel.size()), "sweep order");
    owned.push_back(d_sweep_rel);
    GB_CU(cudaMemcpy(d_sweep_rel, rel.data(), sizeof(uint16_t) * rel.size(),
                     cudaMemcpyHostToDevice), "sweep order");
  }
  {
    // the sync-free sweeps' tables: every row's off-node segments, the
    // tickets of both sweeps, and the column indices in sweep order
    const int Tr = L.energy ? L.dim : -1;
    std::vector<longlong2> sl(N), su(N);
    for (int n = 0; n < LP->num_nodes; n++) {
      const int f0 = LP->fu[n], nr = LP->fu[n + 1] - f0;
      for (int r = 0; r < nr; r++) {
        const int i = f0 + r;
        auto b = LP->colidx.begin() + LP->rowptr[i], e = LP->colidx.begin() + LP->rowptr[i + 1];
        const int64_t di = (int64_t)(std::lower_bound(b, e, i) - LP->colidx.begin());
        const int na = (r == Tr ? L.nvn : nr) - 1 - r;
        sl[i] = make_longlong2(LP->rowptr[i], di - r);
        su[i] = make_longlong2(di + 1 + na, LP->rowptr[i + 1]);
      }
    }
    // one warp per node when every node has at most kWarpMaxRows rows and
    // every row's off-node segments fit its lane group's prefetch window
    {
      bool fits = true;
      for (int n = 0; n < LP->num_nodes && fits; n++) {
        const int f0 = LP->fu[n], nr = LP->fu[n + 1] - f0;
        int R = 1;
        while (R < nr) R <<= 1;
        const int64_t cap = (int64_t)(32 / R) * kPrefetchW;
        if (nr > kWarpMaxRows) fits = false;
        for (int r = 0; r < nr && fits; r++)
          if (sl[f0 + r].y - sl[f0 + r].x > cap || su[f0 + r].y - su[f0 + r].x > cap) fits = false;
      }
      // FP32 sweeps take the warp form whenever it fits; FP64 ones only when
      // the levels are wide (several independent problems interleaved), as
      // the FP64 warp form's 85 registers a thread cost more than its
      // shorter critical path saves on a single mesh
      warp_sweep32 = fits;
      warp_sweep64 = fits && LP->num_nodes > 300LL * (int64_t)lo_ptr.size();
    }
    auto ticks = [&](const std::vector<int> &order, bool upper) {
      std::vector<longlong2> tk(order.size());
      for (size_t t = 0; t < order.size(); t++) {
        const int n = order[t], f0 = LP->fu[n];
        const long long nr = LP->fu[n + 1] - f0;
        tk[t] = make_longlong2((nr << 32) | (long long)f0, ip[n] + (upper ? nr * nr : 0));
      }
      return tk;
    };
    auto upv = [&](const auto &vec, auto **dst, const char *what) -> int {
      GB_CU(cudaMalloc((void **)dst, sizeof(vec[0]) * vec.size()), what);
      owned.push_back(*dst);
      GB_CU(cudaMemcpy(*dst, vec.data(), sizeof(vec[0]) * vec.size(), cudaMemcpyHostToDevice),
            what);
      return 0;
    };
    if (upv(sl, &d_segL, "sweep segments") || upv(su, &d_segU, "sweep segments") ||
        upv(ticks(S.lo_nodes, false), &d_tick_lo, "sweep tickets") ||
        upv(ticks(S.up_nodes, true), &d_tick_up, "sweep tickets"))
      return -1;
    {
      std::vector<int> rev(S.lo_nodes.rbegin(), S.lo_nodes.rend());
      if (upv(ticks(rev, false), &d_tick_lo_rev, "sweep tickets")) return -1;
    }
    GB_CU(cudaMalloc(&d_sweep_cols, sizeof(int) * (size_t)nnz), "sweep columns");
    owned.push_back(d_sweep_cols);
    GB_CU(cudaMemset(d_sweep_cols, 0, sizeof(int) * (size_t)nnz), "sweep columns");
    sweep_gather_kernel<int><<<(N + 7) / 8, 256>>>(N, d_segL, d_segU, d_sweep_rel, P.colidx,
                                                   d_sweep_cols);
    GB_CU(cudaGetLastError(), "sweep columns");
    GB_CU(cudaDeviceSynchronize(), "sweep columns");
  }
  GB_CU(cudaMalloc(&d_lo_nodes, sizeof(int) * S.lo_nodes.size()), "sched");
  GB_CU(cudaMemcpy(d_lo_nodes, S.lo_nodes.data(), sizeof(int) * S.lo_nodes.size(),
                   cudaMemcpyHostToDevice), "sched");
  GB_CU(cudaMalloc(&d_up_nodes, sizeof(int) * S.up_nodes.size()), "sched");
  GB_CU(cudaMemcpy(d_up_nodes, S.up_nodes.data(), sizeof(int) * S.up_nodes.size(),
                   cudaMemcpyHostToDevice), "sched");
  d_fu = c->d_fu;
  if (L.nvn + L.npres > kMaxNodeDofs) return fail("ILU(0) supports at most 16 unknowns per node");
  maxnb = 0;
  lmax = 0;
  for (int n = 0; n < LP->num_nodes; n++) {
    const int nb = LP->nbr_ptr[n + 1] - LP->nbr_ptr[n];
    maxnb = std::max(maxnb, nb);
    const int q = LP->nbr_node[LP->nbr_ptr[n + 1] - 1];
    lmax = std::max(lmax, LP->nbr_off[LP->nbr_ptr[n + 1] - 1] + LP->fu[q + 1] - LP->fu[q]);
  }
  {
    const size_t sm64 = ilu_smem_bytes(sizeof(double), maxnb, L.nvn + L.npres, lmax);
    const size_t sm32 = ilu_smem_bytes(sizeof(float), maxnb, L.nvn + L.npres, lmax);
    if (sm64 > 200 * 1024) return fail("ILU(0) block row does not fit in shared memory");
    GB_CU(cudaFuncSetAttribute(ilu0_block_kernel<double>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm64), "smem");
    GB_CU(cudaFuncSetAttribute(ilu0_block_kernel<float>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm32), "smem");
  }
  GB_CU(cudaMalloc(&d_lu, sizeof(double) * nnz), "ILU factors");
  GB_CU(cudaMalloc(&d_scale, sizeof(double) * N), "scale");
  const size_t wk = (size_t)(kRedBlocks * 3 + (krylov + 2) * kMdBlocks + 4 * (krylov + 2) + 96);
  GB_CU(cudaMalloc(&d_work, sizeof(double) * wk), "work");
  GB_CU(cudaMallocHost(&h_work, sizeof(double) * 4 * (krylov + 2) + 64 * sizeof(double)), "host");
  GB_CU(cudaMalloc(&d_V, sizeof(double) * (size_t)(krylov + 1) * N), "Krylov basis");
  GB_CU(cudaMalloc(&d_t, sizeof(double) * N), "t");
  GB_CU(cudaMalloc(&d_w, sizeof(double) * N), "w");
  GB_CU(cudaMalloc(&d_r, sizeof(double) * N), "r");
  GB_CU(cudaMalloc(&d_xs, sizeof(double) * N), "xs");
  // independent diagonal blocks: node n closes a block when no node up to n
  // has a neighbour beyond n (the graph is symmetric)
  {
    seg_ptr.assign(1, 0);
    int reach = 0;
    for (int n = 0; n < L.num_nodes; n++) {
      reach = std::max(reach, L.nbr_node[L.nbr_ptr[n + 1] - 1]);
      if (reach <= n) seg_ptr.push_back(L.fu[n + 1]);
    }
    nseg = (int)seg_ptr.size() - 1;
  }
  if (nseg > 1) {
    constexpr int64_t kTile = 2048;
    std::vector<int> tseg, tptr(1, 0);
    std::vector<int64_t> tbeg, tend;
    for (int sg = 0; sg < nseg; sg++) {
      for (int64_t u = seg_ptr[sg]; u < seg_ptr[sg + 1]; u += kTile) {
        tseg.push_back(sg);
        tbeg.push_back(u);
        tend.push_back(std::min(seg_ptr[sg + 1], u + kTile));
      }
      tptr.push_back((int)tseg.size());
    }
    ntiles = (int)tseg.size();
    auto upv = [&](auto &vec, auto **dst) -> int {
      GB_CU(cudaMalloc((void **)dst, sizeof(vec[0]) * vec.size()), "segments");
      owned.push_back(*dst);
      GB_CU(cudaMemcpy(*dst, vec.data(), sizeof(vec[0]) * vec.size(), cudaMemcpyHostToDevice),
            "segments");
      return 0;
    };
    if (upv(tseg, &d_tile_seg) || upv(tptr, &d_tile_ptr) || upv(tbeg, &d_tile_beg) ||
        upv(tend, &d_tile_end))
      return -1;
    GB_CU(cudaMalloc(&d_segpart, sizeof(double) * 32 * ntiles), "segments");
    owned.push_back(d_segpart);
    GB_CU(cudaMalloc(&d_segout, sizeof(double) * 3 * 32 * nseg), "segments");
    owned.push_back(d_segout);
    GB_CU(cudaMalloc(&d_segcoef, sizeof(double) * 32 * nseg), "segments");
    owned.push_back(d_segcoef);
    GB_CU(cudaMalloc(&d_segactive, sizeof(int) * nseg), "segments");
    owned.push_back(d_segactive);
    GB_CU(cudaMallocHost(&h_segout, sizeof(double) * 3 * 32 * nseg), "segments");
  }
  return 0;
}

static int lanes_per_row(const Layout &L) {
  const double avg = (double)L.nnz / std::max(1, L.N);
  return avg >= 192 ? 32 : (avg >= 48 ? 16 : 8);
}

template <class T>
static cudaError_t spmv(const Context *C, int lpr, const T *vals, const T *x, T *y, cudaStream_t st) {
  // FP64: 8 lanes a row.  On GB300 the FP64 product is bound by the FP64
  // pipe as much as by HBM (ncu: pipe 89 % busy at 32 lanes a row, half of it
  // the shuffle-reduction adds); 8 lanes cut those adds to a sixth.
  if (sizeof(T) == 8) lpr = 8;
  const int N = C->L.N, threads = 256;
  const int blocks = (int)(((int64_t)N * lpr + threads - 1) / threads);
  switch (lpr) {
  case 32: spmv_kernel<T, 32><<<blocks, threads, 0, st>>>(N, C->d_rowptr, C->d_colidx, vals, x, y); break;
  case 16: spmv_kernel<T, 16><<<blocks, threads, 0, st>>>(N, C->d_rowptr, C->d_colidx, vals, x, y); break;
  default: spmv_kernel<T, 8><<<blocks, threads, 0, st>>>(N, C->d_rowptr, C->d_colidx, vals, x, y);
  }
  return cudaGetLastError();
}

template <class T>
static cudaError_t capture_prec(Solver *S, const T *lu, const T *binv, T *z, cudaStream_t st,
                                cudaGraphExec_t *out) {
  cudaGraph_t g;
  const TrsvArgs a = trsv_args(S);
  cudaError_t e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  for (size_t l = 0; l + 1 < S->lo_ptr.size(); l++) {
    const int cnt = S->lo_ptr[l + 1] - S->lo_ptr[l];
    trsv_level_cta_kernel<T, true><<<cnt, kTrsvThreads, 0, st>>>(S->d_lo_nodes + S->lo_ptr[l], a,
                                                                 lu, binv, z);
  }
  for (size_t l = 0; l + 1 < S->up_ptr.size(); l++) {
    const int cnt = S->up_ptr[l + 1] - S->up_ptr[l];
    trsv_level_cta_kernel<T, false><<<cnt, kTrsvThreads, 0, st>>>(S->d_up_nodes + S->up_ptr[l],
                                                                  a, lu, binv, z);
  }
  e = cudaStreamEndCapture(st, &g);
  if (e != cudaSuccess) return e;
  e = cudaGraphInstantiate(out, g, 0);
  cudaGraphDestroy(g);
  return e;
}

int Solver::factor(const double *vals, bool fp32, cudaStream_t st) {
  d_A = vals;
  int *nfix = (int *)(d_work + kRedBlocks * 3 + 10);
  GB_CU(cudaMemsetAsync(nfix, 0, sizeof(int), st), "pivot count");
  const Layout &L = C->L;
  IluArgs g;
  g.fu = P.fu;
  g.rowptr = P.rowptr;
  g.nbr_ptr = P.nbr_ptr;
  g.nbr_node = P.nbr_node;
  g.nbr_off = P.nbr_off;
  g.nbr_offT = P.nbr_offT;
  g.nbr_self = P.nbr_self;
  g.dim = L.dim;
  g.nvn = L.nvn;
  g.energy = L.energy;
  g.maxnb = maxnb;
  g.lmax = lmax;
  g.maxnr = L.nvn + L.npres;
  g.tau = pivot_tau;
  g.nfix = nfix;
  if (fp32 && !d_lu32) {
    GB_CU(cudaMalloc(&d_lu32, sizeof(float) * nnz), "ILU32");
    GB_CU(cudaMalloc(&d_a32, sizeof(float) * nnz), "A32");
    GB_CU(cudaMalloc(&d_V32, sizeof(float) * (size_t)(max_krylov + 1) * N), "V32");
    GB_CU(cudaMalloc(&d_t32, sizeof(float) * N), "t32");
    GB_CU(cudaMalloc(&d_w32, sizeof(float) * N), "w32");
    if (ordering == 1) {
      GB_CU(cudaMalloc(&d_tp32, sizeof(float) * N), "permuted vector");
      owned.push_back(d_tp32);
    }
  }
  const double *Af = vals;  // the matrix the factors are built from
  if (ordering == 1) {
    gather_kernel<double><<<1216, 256, 0, st>>>(nnz, d_vmap, vals, d_Ap);
    GB_CU(cudaGetLastError(), "matrix permutation");
    Af = d_Ap;
  }
  for (size_t l = 0; l + 1 < lo_ptr.size(); l++) {
    const int cnt = lo_ptr[l + 1] - lo_ptr[l];
    if (fp32) {
      const size_t sm = ilu_smem_bytes(sizeof(float), maxnb, g.maxnr, lmax);
      ilu0_block_kernel<float><<<cnt, 256, sm, st>>>(d_lo_nodes + lo_ptr[l], g, Af, d_lu32);
    } else {
      const size_t sm = ilu_smem_bytes(sizeof(double), maxnb, g.maxnr, lmax);
      ilu0_block_kernel<double><<<cnt, 256, sm, st>>>(d_lo_nodes + lo_ptr[l], g, Af, d_lu);
    }
  }
  GB_CU(cudaGetLastError(), "ILU(0) factorisation");
  {
    const TrsvArgs a = trsv_args(this);
    const int gs = (N + 7) / 8;
    if (fp32) {
      if (!d_binv32) GB_CU(cudaMalloc(&d_binv32, sizeof(float) * inv_len), "block inverses");
      if (!d_lus32) GB_CU(cudaMalloc(&d_lus32, sizeof(float) * nnz), "sweep-ordered factors");
      block_inverse_kernel<float><<<(C->L.num_nodes + 7) / 8, 256, 0, st>>>(a, d_lu32, d_binv32);
      sweep_gather_kernel<float><<<gs, 256, 0, st>>>(N, d_segL, d_segU, d_sweep_rel, d_lu32,
                                                     d_lus32);
    } else {
      if (!d_lus) GB_CU(cudaMalloc(&d_lus, sizeof(double) * nnz), "sweep-ordered factors");
      block_inverse_kernel<double><<<(C->L.num_nodes + 7) / 8, 256, 0, st>>>(a, d_lu, d_binv);
      sweep_gather_kernel<double><<<gs, 256, 0, st>>>(N, d_segL, d_segU, d_sweep_rel, d_lu,
                                                      d_lus);
    }
    GB_CU(cudaGetLastError(), "block inverses");
  }
  if (fp32) {
    to_f32_kernel<<<1216, 256, 0, st>>>(nnz, vals, d_a32);
    GB_CU(cudaGetLastError(), "FP32 matrix copy");
    if (!prec32 && use_level_graph())
      GB_CU(capture_prec<float>(this, d_lu32, d_binv32, ordering ? d_tp32 : d_t32, st, &prec32),
            "ILU32 graph");
    have_lu32 = true;
  } else {
    if (!prec64 && use_level_graph())
      GB_CU(capture_prec<double>(this, d_lu, d_binv, ordering ? d_tp : d_t, st, &prec64),
            "ILU graph");
    have_lu64 = true;
  }
  return 0;
}

int Solver::refresh(const double *vals, bool fp32, cudaStream_t st) {
  if (!has_factors(fp32)) return fail("no ILU(0) factors to reuse");
  d_A = vals;
  if (fp32) {
    to_f32_kernel<<<1216, 256, 0, st>>>(nnz, vals, d_a32);
    GB_CU(cudaGetLastError(), "FP32 matrix copy");
  }
  return 0;
}

int Solver::copy_factors(double *host, bool fp32, cudaStream_t st) {
  const int64_t nnz = C->L.nnz;
  if (ordering != 0) return fail("the factors are in the multicoloured order");
  GB_CU(cudaStreamSynchronize(st), "factor");
  if (fp32) {
    std::vector<float> tmp((size_t)nnz);
    GB_CU(cudaMemcpy(tmp.data(), d_lu32, sizeof(float) * nnz, cudaMemcpyDeviceToHost),
          "factor copy");
    for (int64_t k = 0; k < nnz; k++) host[k] = tmp[(size_t)k];
  } else {
    GB_CU(cudaMemcpy(host, d_lu, sizeof(double) * nnz, cudaMemcpyDeviceToHost), "factor copy");
  }
  return 0;
}

template <class T>
static int sync_free_apply(Solver *S, const T *lus, const T *binv, T *z, cudaStream_t st) {
  if (!S->d_flags) {
    GB_CU(cudaMalloc(&S->d_flags, 16 * sizeof(unsigned)), "trsv error word");
    GB_CU(cudaMemsetAsync(S->d_flags, 0, 16 * sizeof(unsigned), st), "trsv error word");
    GB_CU(cudaMalloc(&S->d_sweep_y, sizeof(double) * (size_t)S->N), "trsv scratch");
    int per_sm = 1 << 30, dev = 0, sms = 0;
    const void *fns[4] = {(const void *)trsv_sync_free_kernel<double, true>,
                          (const void *)trsv_sync_free_kernel<double, false>,
                          (const void *)trsv_sync_free_kernel<float, true>,
                          (const void *)trsv_sync_free_kernel<float, false>};
    const void *wfns[4] = {(const void *)trsv_sync_free_warp_kernel<double, true>,
                           (const void *)trsv_sync_free_warp_kernel<double, false>,
                           (const void *)trsv_sync_free_warp_kernel<float, true>,
                           (const void *)trsv_sync_free_warp_kernel<float, false>};
    int wper_sm = 1 << 30;
    for (const void *f : fns) {
      int b = 0;
      GB_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, f, kTrsvThreads, 0), "occupancy");
      per_sm = std::min(per_sm, b);
    }
    for (const void *f : wfns) {
      int b = 0;
      GB_CU(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, f, kWarpSweepThreads, 0),
            "occupancy");
      wper_sm = std::min(wper_sm, b);
    }
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    S->trsv_grid = std::max(1, per_sm) * sms;
    S->trsv_grid_warp = std::max(1, wper_sm) * sms;
    S->prep_grid = 2 * sms;
  }
  TrsvArgs g = trsv_args(S);  // the tickets and segments are set per sweep below
  g.error = (int *)(S->d_flags + 4);
  g.cols = S->d_sweep_cols;
  T *y = static_cast<T *>(S->d_sweep_y);
  // the host-injected fault of gb_set_sweep_fault: the lower sweep's nodes in
  // reverse order (every dependency after its dependant) on one CTA, whose
  // first wait can then only end by running out
  const longlong2 *lo_tick = S->d_tick_lo;
  const bool warp = sizeof(T) == 4 ? S->warp_sweep32 : S->warp_sweep64;
  int grid = warp ? S->trsv_grid_warp : S->trsv_grid;
  if (S->C->sweep_reverse_lower) {
    lo_tick = S->d_tick_lo_rev;
    grid = 1;
  }
  // L: z -> y, then U: y -> z; each output starts all unpublished
  trsv_prepare_kernel<T><<<S->prep_grid, 256, 0, st>>>(S->N, y);
  g.tick = lo_tick;
  g.seg = S->d_segL;
  if (warp)
    trsv_sync_free_warp_kernel<T, true><<<grid, kWarpSweepThreads, 0, st>>>(g, lus, binv, z, y);
  else
    trsv_sync_free_kernel<T, true><<<grid, kTrsvThreads, 0, st>>>(g, lus, binv, z, y);
  trsv_prepare_kernel<T><<<S->prep_grid, 256, 0, st>>>(S->N, z);
  g.tick = S->d_tick_up;
  g.seg = S->d_segU;
  if (warp)
    trsv_sync_free_warp_kernel<T, false><<<grid, kWarpSweepThreads, 0, st>>>(g, lus, binv, y, z);
  else
    trsv_sync_free_kernel<T, false><<<grid, kTrsvThreads, 0, st>>>(g, lus, binv, y, z);
  GB_CU(cudaGetLastError(), "trsv");
  return 0;
}

bool Solver::use_level_graph() const {
  return C->trsv == 1 || (C->trsv == 2 && num_levels <= kMaxGraphLevels);
}

int Solver::check_trsv_error() {
  if (!d_flags) return 0;
  int h = 0;
  GB_CU(cudaMemcpy(&h, d_flags + 4, sizeof(int), cudaMemcpyDeviceToHost), "trsv error");
  if (h) {
    cudaMemset(d_flags + 4, 0, sizeof(int));
    return fail("triangular solve: a dependency wait gave up");
  }
  return 0;
}

template <class T>
static int apply_prec(Solver *S, const T *lus, const T *binv, T *t, T *tp,
                      cudaGraphExec_t graph, cudaStream_t st) {
  T *z = t;
  if (S->ordering == 1) {  // t -> P t, solve, P^T
    gather_kernel<T><<<304, 256, 0, st>>>(S->N, S->d_umap, t, tp);
    z = tp;
  }
  if (!S->use_level_graph()) {
    if (sync_free_apply<T>(S, lus, binv, z, st)) return -1;
  } else {
    GB_CU(cudaGraphLaunch(graph, st), "ILU apply");
  }
  if (S->ordering == 1) scatter_kernel<T><<<304, 256, 0, st>>>(S->N, S->d_umap, tp, t);
  GB_CU(cudaGetLastError(), "ILU apply");
  return 0;
}

int Solver::apply_prec64(cudaStream_t st) {
  return apply_prec<double>(this, d_lus, d_binv, d_t, d_tp, prec64, st);
}
int Solver::apply_prec32(cudaStream_t st) {
  return apply_prec<float>(this, d_lus32, d_binv32, d_t32, d_tp32, prec32, st);
}

// ------------------------------------------------------------ helpers

int device_norms(Context *C, const double *x, int n, double out3[3], cudaStream_t st) {
  Solver &S = *C->solver;
  norms_partial_kernel<double><<<kRedBlocks, kRedThreads, 0, st>>>(n, x, S.d_work);
  norms_final_kernel<<<1, 32, 0, st>>>(kRedBlocks, S.d_work, S.d_work + kRedBlocks * 3);
  GB_CU(cudaGetLastError(), "norms");
  GB_CU(cudaMemcpyAsync(S.h_work, S.d_work + kRedBlocks * 3, 3 * sizeof(double),
                        cudaMemcpyDeviceToHost, st), "norms copy");
  GB_CU(cudaStreamSynchronize(st), "norms sync");
  memcpy(out3, S.h_work, 3 * sizeof(double));
  return 0;
}

int row_sum_scale(Context *C, double *vals, double *R, cudaStream_t st) {
  Solver &S = *C->solver;
  const int N = C->L.N;
  int *zr = (int *)(S.d_work + kRedBlocks * 3 + 8);
  GB_CU(cudaMemsetAsync(zr, 0, sizeof(int), st), "scale");
  row_sum_scale_kernel<<<(int)(((int64_t)N * 32 + 255) / 256), 256, 0, st>>>(
      N, C->d_rowptr, S.d_diag, vals, R, S.d_scale, zr);
  GB_CU(cudaGetLastError(), "row sum scaling");
  return 0;
}

// GMRES(m), right preconditioned.  T = double: FP64 throughout; T = float:
// FP32 matrix, factors and vectors (sums in FP64).  Solves A x = b with b,
// x of type T on the device, x = 0 on entry; stops when the preconditioned
// system's true residual <= tol * ||b|| or after maxit iterations.
template <class T>
static int gmres(Context *C, const T *b, T *x, double tol, int maxit, int m, int *its,
                 double *relres, cudaStream_t st, bool flexible = false) {
  Solver &S = *C->solver;
  const Layout &L = C->L;
  const int N = L.N, lpr = lanes_per_row(L);
  const bool f32 = sizeof(T) == 4;
  T *V = f32 ? (T *)S.d_V32 : (T *)S.d_V;
  T *t = f32 ? (T *)S.d_t32 : (T *)S.d_t;
  T *w = f32 ? (T *)S.d_w32 : (T *)S.d_w;
  const T *A = f32 ? (const T *)S.d_a32 : (const T *)S.d_A;
  const int64_t ld = N;
  double *dred = S.d_work;                           // partials
  double *dh = S.d_work + kRedBlocks * 3 + 16;       // (m+2) results
  double *dpart = dh + (m + 2) * 2 + 8;              // (m+2) * kMdBlocks
  // the row-parallel kernels (w -= V h, y = V c) get a thread per unknown:
  // enough loads in flight to stream the basis at HBM speed
  const int rows_grid = (N + kRedThreads - 1) / kRedThreads;
  double *hh = S.h_work;
  std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1), y(m);
  auto norm = [&](const T *v, double *out) -> int {
    norms_partial_kernel<T><<<kRedBlocks, kRedThreads, 0, st>>>(N, v, dred);
    norms_final_kernel<<<1, 32, 0, st>>>(kRedBlocks, dred, dh);
    GB_CU(cudaMemcpyAsync(hh, dh, sizeof(double), cudaMemcpyDeviceToHost, st), "norm");
    GB_CU(cudaStreamSynchronize(st), "norm sync");
    *out = hh[0];
    return 0;
  };
  GB_CU(cudaMemsetAsync(x, 0, sizeof(T) * N, st), "x0");
  double bnorm;
  if (norm(b, &bnorm)) return -1;
  *its = 0;
  *relres = 0.0;
  if (bnorm == 0.0) return 0;
  // r = b (x = 0)
  GB_CU(cudaMemcpyAsync(V, b, sizeof(T) * N, cudaMemcpyDeviceToDevice, st), "r0");
  double beta = bnorm;
  int total = 0;
  while (true) {
    // V0 = r / beta (dh[0] = beta)
    hh[0] = beta;
    GB_CU(cudaMemcpyAsync(dh, hh, sizeof(double), cudaMemcpyHostToDevice, st), "beta");
    scale_copy_kernel<T><<<kRedBlocks, kRedThreads, 0, st>>>(N, V, dh, V);
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    bool done = false;
    for (; j < m && total < maxit; j++) {
      const T *zj = t;  // M^-1 v_j
      if constexpr (std::is_same<T, double>::value) {
        if (flexible) {
          // the preconditioner in FP32: v_j -> FP32, sweeps, z_j kept in FP64
          to_f32_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(N, V + j * ld, S.d_t32);
          if (S.apply_prec32(st)) return -1;
          to_f64_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(N, S.d_t32, S.d_Z + j * ld);
          zj = S.d_Z + j * ld;
        }
      }
      if (!flexible) {
        GB_CU(cudaMemcpyAsync(t, V + j * ld, sizeof(T) * N, cudaMemcpyDeviceToDevice, st), "t");
        if (f32 ? S.apply_prec32(st) : S.apply_prec64(st)) return -1;
      }
      GB_CU(spmv<T>(C, lpr, A, zj, w, st), "spmv");
      // CGS2 on the device; the host reads both passes and the norm in one copy
      std::vector<double> hcol(j + 2, 0.0);
      double *dh1 = dh, *dh2 = dh + (m + 2), *dnrm = dh + 2 * (m + 2);
      multidot_tile_kernel<T><<<dim3(kMdBlocks, (j + kMdCols) / kMdCols), kRedThreads, 0, st>>>(
          N, j + 1, V, ld, w, dpart);
      // a warp per coefficient, eight a block
      const int fin = (j + 1 + 7) / 8;
      multidot_final_kernel<<<fin, 256, 0, st>>>(j + 1, kMdBlocks, dpart, dh1);
      gemv_sub_kernel<T><<<rows_grid, kRedThreads, 0, st>>>(N, j + 1, V, ld, dh1, w);
      multidot_tile_kernel<T><<<dim3(kMdBlocks, (j + kMdCols) / kMdCols), kRedThreads, 0, st>>>(
          N, j + 1, V, ld, w, dpart);
      multidot_final_kernel<<<fin, 256, 0, st>>>(j + 1, kMdBlocks, dpart, dh2);
      gemv_sub_kernel<T><<<rows_grid, kRedThreads, 0, st>>>(N, j + 1, V, ld, dh2, w);
      norms_partial_kernel<T><<<kRedBlocks, kRedThreads, 0, st>>>(N, w, dred);
      norms_final_kernel<<<1, 32, 0, st>>>(kRedBlocks, dred, dnrm);
      scale_copy_kernel<T><<<kRedBlocks, kRedThreads, 0, st>>>(N, w, dnrm, V + (j + 1) * ld);
      GB_CU(cudaGetLastError(), "Arnoldi step");
      GB_CU(cudaMemcpyAsync(hh, dh, sizeof(double) * (2 * (m + 2) + 1), cudaMemcpyDeviceToHost,
                            st), "h");
      GB_CU(cudaStreamSynchronize(st), "h sync");
      for (int i = 0; i <= j; i++) hcol[i] = hh[i] + hh[(m + 2) + i];
      const double hn = hh[2 * (m + 2)];
      hcol[j + 1] = hn;
      total++;
      // Givens
      for (int i = 0; i < j; i++) {
        const double a = cs[i] * hcol[i] + sn[i] * hcol[i + 1];
        hcol[i + 1] = -sn[i] * hcol[i] + cs[i] * hcol[i + 1];
        hcol[i] = a;
      }
      const double den = std::hypot(hcol[j], hcol[j + 1]);
      cs[j] = den == 0.0 ? 1.0 : hcol[j] / den;
      sn[j] = den == 0.0 ? 0.0 : hcol[j + 1] / den;
      hcol[j] = den;
      hcol[j + 1] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      for (int i = 0; i <= j; i++) H[(size_t)i * m + j] = hcol[i];
      if (std::fabs(g[j + 1]) <= tol * bnorm || hn == 0.0) {
        j++;
        done = true;
        break;
      }
    }
    // y = H^-1 g, x += M^-1 V y
    for (int i = j - 1; i >= 0; i--) {
      double sum = g[i];
      for (int k = i + 1; k < j; k++) sum -= H[(size_t)i * m + k] * y[k];
      y[i] = H[(size_t)i * m + i] != 0.0 ? sum / H[(size_t)i * m + i] : 0.0;
    }
    memcpy(hh, y.data(), sizeof(double) * j);
    GB_CU(cudaMemcpyAsync(dh, hh, sizeof(double) * j, cudaMemcpyHostToDevice, st), "y");
    if constexpr (std::is_same<T, double>::value) {
      // flexible: x += Z y, the preconditioned vectors as they were applied
      if (flexible) gemv_kernel<T><<<rows_grid, kRedThreads, 0, st>>>(N, j, S.d_Z, ld, dh, t);
    }
    if (!flexible) {
      gemv_kernel<T><<<rows_grid, kRedThreads, 0, st>>>(N, j, V, ld, dh, t);
      if (f32 ? S.apply_prec32(st) : S.apply_prec64(st)) return -1;
    }
    add_kernel<T><<<kRedBlocks, kRedThreads, 0, st>>>(N, t, x);
    // true residual r = b - A x into V0
    GB_CU(spmv<T>(C, lpr, A, x, V, st), "spmv");
    sub_from_kernel<T><<<kRedBlocks, kRedThreads, 0, st>>>(N, b, V);
    if (norm(V, &beta)) return -1;
    *its = total;
    *relres = beta / bnorm;
    if (beta <= tol * bnorm || total >= maxit || (done && beta <= 10 * tol * bnorm)) break;
  }
  return 0;
}

// ------------------------------------------------------------ batched GMRES
//
// Independent problems in one matrix (diagonal blocks over contiguous
// unknown ranges): one GMRES per block, run together.  Every inner product
// is segmented -- a tile of <= 2048 unknowns lies in one block; tiles give
// partial sums, one warp per block adds them -- so each block has its own
// Arnoldi coefficients, Hessenberg matrix, Givens rotations, restarts and
// convergence test; SpMV and the (block-diagonal) ILU(0) serve all blocks
// at once.

// part[t][j] = sum over tile t of V_j . w, j < k (k <= 32)
template <class T>
__global__ void seg_dots_kernel(int k, const T *__restrict__ V, int64_t ld,
                                const T *__restrict__ w, const int64_t *__restrict__ tbeg,
                                const int64_t *__restrict__ tend, double *__restrict__ part) {
  __shared__ double red[8];
  const int t = blockIdx.x, lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int64_t b = tbeg[t], e = tend[t];
  using A = acc_t<T>;
  for (int j = 0; j < k; j++) {
    A acc = 0;
    for (int64_t i = b + threadIdx.x; i < e; i += blockDim.x)
      acc = fmx((A)V[j * ld + i], (A)w[i], acc);
    const double sum = warp_sum((double)acc);
    if (lane == 0) red[wp] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); q++) tot += red[q];
      part[(int64_t)t * 32 + j] = tot;
    }
    __syncthreads();
  }
}

// out[s][j] = sum over the tiles of block s of part[t][j]; one warp per block
__global__ void seg_reduce_kernel(int nseg, int k, const int *__restrict__ tptr,
                                  const double *__restrict__ part, double *__restrict__ out) {
  const int sg = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (sg >= nseg) return;
  for (int j = 0; j < k; j++) {
    double sum = 0.0;
    for (int t = tptr[sg] + lane; t < tptr[sg + 1]; t += 32) sum += part[(int64_t)t * 32 + j];
    sum = warp_sum(sum);
    if (lane == 0) out[sg * 32 + j] = sum;
  }
}

// w -= sum_j c[s][j] V_j on block s (c = the reduced dots), or with
// ACCUMULATE = false: y = sum_j c[s][j] V_j
template <class T, bool SUB>
__global__ void seg_gemv_kernel(int k, const T *__restrict__ V, int64_t ld,
                                const double *__restrict__ c, const int *__restrict__ tseg,
                                const int64_t *__restrict__ tbeg, const int64_t *__restrict__ tend,
                                T *__restrict__ y) {
  __shared__ double cs[32];
  const int t = blockIdx.x;
  const int sg = tseg[t];
  if (threadIdx.x < 32) cs[threadIdx.x] = threadIdx.x < k ? c[sg * 32 + threadIdx.x] : 0.0;
  __syncthreads();
  using A = acc_t<T>;
  for (int64_t i = tbeg[t] + threadIdx.x; i < tend[t]; i += blockDim.x) {
    A acc = 0;
    for (int j = 0; j < k; j++) acc = fmx((A)cs[j], (A)V[j * ld + i], acc);
    y[i] = SUB ? (T)((A)y[i] - acc) : (T)acc;
  }
}

// dst = src * alpha[s] on block s; alpha = 1 / sqrt(norm2[s]) for active
// blocks with a nonzero norm, else 0 (from the reduced norms when scale is NULL)
template <class T>
__global__ void seg_scale_kernel(const T *__restrict__ src, const double *__restrict__ norm2,
                                 const int *__restrict__ active, const int *__restrict__ tseg,
                                 const int64_t *__restrict__ tbeg, const int64_t *__restrict__ tend,
                                 T *__restrict__ dst) {
  const int t = blockIdx.x, sg = tseg[t];
  const double n2 = norm2[sg * 32];
  const acc_t<T> a = (acc_t<T>)((active[sg] && n2 > 0.0) ? 1.0 / sqrt(n2) : 0.0);
  for (int64_t i = tbeg[t] + threadIdx.x; i < tend[t]; i += blockDim.x)
    dst[i] = (T)((acc_t<T>)src[i] * a);
}

template <class T>
static int gmres_seg(Context *C, const T *b, T *x, double tol, int maxit, int m, int *its,
                     double *relres, cudaStream_t st,
                     bool flexible = false) {
  Solver &S = *C->solver;
  const Layout &L = C->L;
  const int N = L.N, lpr = lanes_per_row(L), ns = S.nseg, nt = S.ntiles;
  m = std::min(m, 31);
  const bool f32 = sizeof(T) == 4;
  T *V = f32 ? (T *)S.d_V32 : (T *)S.d_V;
  T *t = f32 ? (T *)S.d_t32 : (T *)S.d_t;
  T *w = f32 ? (T *)S.d_w32 : (T *)S.d_w;
  const T *A = f32 ? (const T *)S.d_a32 : (const T *)S.d_A;
  const int64_t ld = N;
  double *o1 = S.d_segout, *o2 = o1 + 32 * ns, *o3 = o2 + 32 * ns;
  double *h1 = S.h_segout, *h2 = h1 + 32 * ns, *h3 = h2 + 32 * ns;
  const int rblocks = (ns + 7) / 8;
  auto dots = [&](int k, const T *Vb, const T *wv, double *out) {
    seg_dots_kernel<T><<<nt, 256, 0, st>>>(k, Vb, ld, wv, S.d_tile_beg, S.d_tile_end,
                                           S.d_segpart);
    seg_reduce_kernel<<<rblocks, 256, 0, st>>>(ns, k, S.d_tile_ptr, S.d_segpart, out);
  };
  std::vector<int> active(ns, 1), done(ns, 0);
  std::vector<double> bnorm(ns), beta(ns), coef(32 * (size_t)ns);
  std::vector<double> H((size_t)ns * (m + 1) * m), cs((size_t)ns * m), sn((size_t)ns * m),
      g((size_t)ns * (m + 1)), y(m);
  std::vector<int> used(ns);
  auto upload_active = [&]() -> int {
    GB_CU(cudaMemcpyAsync(S.d_segactive, active.data(), sizeof(int) * ns, cudaMemcpyHostToDevice,
                          st), "active");
    return 0;
  };
  GB_CU(cudaMemsetAsync(x, 0, sizeof(T) * N, st), "x0");
  dots(1, b, b, o3);
  GB_CU(cudaMemcpyAsync(h3, o3, sizeof(double) * 32 * ns, cudaMemcpyDeviceToHost, st), "norms");
  GB_CU(cudaStreamSynchronize(st), "norms");
  bool any = false;
  for (int sg = 0; sg < ns; sg++) {
    bnorm[sg] = std::sqrt(h3[sg * 32]);
    beta[sg] = bnorm[sg];
    active[sg] = bnorm[sg] > 0.0;
    any |= active[sg] != 0;
  }
  *its = 0;
  *relres = 0.0;
  if (!any) return 0;
  GB_CU(cudaMemcpyAsync(V, b, sizeof(T) * N, cudaMemcpyDeviceToDevice, st), "r0");
  int total = 0;
  while (true) {
    if (upload_active()) return -1;
    // V0 = r / beta per block (o3 holds the squared norms of r)
    seg_scale_kernel<T><<<nt, 256, 0, st>>>(V, o3, S.d_segactive, S.d_tile_seg, S.d_tile_beg,
                                            S.d_tile_end, V);
    for (int sg = 0; sg < ns; sg++) {
      std::fill(&g[(size_t)sg * (m + 1)], &g[(size_t)sg * (m + 1)] + m + 1, 0.0);
      g[(size_t)sg * (m + 1)] = beta[sg];
      done[sg] = active[sg] ? 0 : -1;  // -1: converged before this cycle
      used[sg] = 0;
    }
    int j = 0;
    for (; j < m && total < maxit; j++) {
      const T *zj = t;  // M^-1 v_j
      if constexpr (std::is_same<T, double>::value) {
        if (flexible) {
          // the (block-diagonal) preconditioner in FP32, z_j kept in FP64
          to_f32_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(N, V + j * ld, S.d_t32);
          if (S.apply_prec32(st)) return -1;
          to_f64_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(N, S.d_t32, S.d_Z + j * ld);
          zj = S.d_Z + j * ld;
        }
      }
      if (!flexible) {
        GB_CU(cudaMemcpyAsync(t, V + j * ld, sizeof(T) * N, cudaMemcpyDeviceToDevice, st), "t");
        if (f32 ? S.apply_prec32(st) : S.apply_prec64(st)) return -1;
      }
      GB_CU(spmv<T>(C, lpr, A, zj, w, st), "spmv");
      dots(j + 1, V, w, o1);
      seg_gemv_kernel<T, true><<<nt, 256, 0, st>>>(j + 1, V, ld, o1, S.d_tile_seg,
                                                   S.d_tile_beg, S.d_tile_end, w);
      dots(j + 1, V, w, o2);
      seg_gemv_kernel<T, true><<<nt, 256, 0, st>>>(j + 1, V, ld, o2, S.d_tile_seg,
                                                   S.d_tile_beg, S.d_tile_end, w);
      dots(1, w, w, o3);
      seg_scale_kernel<T><<<nt, 256, 0, st>>>(w, o3, S.d_segactive, S.d_tile_seg, S.d_tile_beg,
                                              S.d_tile_end, V + (j + 1) * ld);
      GB_CU(cudaGetLastError(), "batched Arnoldi step");
      GB_CU(cudaMemcpyAsync(h1, o1, sizeof(double) * 3 * 32 * ns, cudaMemcpyDeviceToHost, st),
            "h");
      GB_CU(cudaStreamSynchronize(st), "h sync");
      total++;
      bool changed = false, all_done = true;
      for (int sg = 0; sg < ns; sg++) {
        if (done[sg] != 0) continue;
        double *Hs = &H[(size_t)sg * (m + 1) * m], *gs = &g[(size_t)sg * (m + 1)];
        double *csg = &cs[(size_t)sg * m], *sng = &sn[(size_t)sg * m];
        double hcol[33];
        for (int i = 0; i <= j; i++) hcol[i] = h1[sg * 32 + i] + h2[sg * 32 + i];
        const double hn = std::sqrt(h3[sg * 32]);
        hcol[j + 1] = hn;
        for (int i = 0; i < j; i++) {
          const double a = csg[i] * hcol[i] + sng[i] * hcol[i + 1];
          hcol[i + 1] = -sng[i] * hcol[i] + csg[i] * hcol[i + 1];
          hcol[i] = a;
        }
        const double den = std::hypot(hcol[j], hcol[j + 1]);
        csg[j] = den == 0.0 ? 1.0 : hcol[j] / den;
        sng[j] = den == 0.0 ? 0.0 : hcol[j + 1] / den;
        hcol[j] = den;
        gs[j + 1] = -sng[j] * gs[j];
        gs[j] = csg[j] * gs[j];
        for (int i = 0; i <= j; i++) Hs[(size_t)i * m + j] = hcol[i];
        used[sg] = j + 1;
        if (std::fabs(gs[j + 1]) <= tol * bnorm[sg] || hn == 0.0) {
          done[sg] = 1;
          active[sg] = 0;
          changed = true;
        } else {
          all_done = false;
        }
      }
      if (changed && upload_active()) return -1;
      if (all_done) {
        j++;
        break;
      }
    }
    // x += M^-1 sum_j y_j V_j, block by block
    std::fill(coef.begin(), coef.end(), 0.0);
    int kmax = 0;
    for (int sg = 0; sg < ns; sg++) {
      const int js = used[sg];
      if (js == 0) continue;
      const double *Hs = &H[(size_t)sg * (m + 1) * m], *gs = &g[(size_t)sg * (m + 1)];
      for (int i = js - 1; i >= 0; i--) {
        double sum = gs[i];
        for (int k2 = i + 1; k2 < js; k2++) sum -= Hs[(size_t)i * m + k2] * y[k2];
        y[i] = Hs[(size_t)i * m + i] != 0.0 ? sum / Hs[(size_t)i * m + i] : 0.0;
      }
      for (int i = 0; i < js; i++) coef[(size_t)sg * 32 + i] = y[i];
      kmax = std::max(kmax, js);
    }
    if (kmax > 0) {
      GB_CU(cudaMemcpyAsync(S.d_segcoef, coef.data(), sizeof(double) * 32 * ns,
                            cudaMemcpyHostToDevice, st), "y");
      if constexpr (std::is_same<T, double>::value) {
        // flexible: x += Z y, the preconditioned vectors as they were applied
        if (flexible)
          seg_gemv_kernel<T, false><<<nt, 256, 0, st>>>(kmax, S.d_Z, ld, S.d_segcoef,
                                                        S.d_tile_seg, S.d_tile_beg,
                                                        S.d_tile_end, t);
      }
      if (!flexible) {
        seg_gemv_kernel<T, false><<<nt, 256, 0, st>>>(kmax, V, ld, S.d_segcoef, S.d_tile_seg,
                                                      S.d_tile_beg, S.d_tile_end, t);
        if (f32 ? S.apply_prec32(st) : S.apply_prec64(st)) return -1;
      }
      add_kernel<T><<<kRedBlocks, kRedThreads, 0, st>>>(N, t, x);
    }
    // true residual per block
    GB_CU(spmv<T>(C, lpr, A, x, V, st), "spmv");
    sub_from_kernel<T><<<kRedBlocks, kRedThreads, 0, st>>>(N, b, V);
    dots(1, V, V, o3);
    GB_CU(cudaMemcpyAsync(h3, o3, sizeof(double) * 32 * ns, cudaMemcpyDeviceToHost, st), "norms");
    GB_CU(cudaStreamSynchronize(st), "norms");
    double worst = 0.0;
    bool all_conv = true;
    for (int sg = 0; sg < ns; sg++) {
      if (bnorm[sg] == 0.0) {
        active[sg] = 0;
        continue;
      }
      beta[sg] = std::sqrt(h3[sg * 32]);
      const bool conv = beta[sg] <= tol * bnorm[sg];
      active[sg] = !conv;
      all_conv &= conv;
      worst = std::max(worst, beta[sg] / bnorm[sg]);
    }
    *its = total;
    *relres = worst;
    if (all_conv || total >= maxit) break;
  }
  return 0;
}

// Solves the scaled system A dx = R (both on the device, A = d_vals_scaled
// after factorisation).  FP64: GMRES in FP64.  FP32 refined: FP32 GMRES on
// the normalised residual inside FP64 iterative refinement.
static int linear_solve_impl(Context *C, const double *R, double *dx, const LinearOpts &o,
                             LinearStats *s, cudaStream_t st);

int linear_solve(Context *C, const double *R, double *dx, const LinearOpts &o, LinearStats *s,
                 cudaStream_t st) {
  const int rc = linear_solve_impl(C, R, dx, o, s, st);
  cudaError_t e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(e, "linear solve");
  if (C->solver->check_trsv_error()) return -1;
  return rc;
}

static int linear_solve_impl(Context *C, const double *R, double *dx, const LinearOpts &o,
                             LinearStats *s, cudaStream_t st) {
  Solver &S = *C->solver;
  const int N = C->L.N;
  s->iterations = 0;
  s->refinements = 0;
  if (o.fp32_prec) {
    if (!S.d_Z) GB_CU(cudaMalloc(&S.d_Z, sizeof(double) * (size_t)S.max_krylov * N), "Z basis");
    int its;
    double rr;
    if (S.nseg > 1 ? gmres_seg<double>(C, R, dx, o.tol, o.maxit, o.krylov, &its, &rr, st, true)
                   : gmres<double>(C, R, dx, o.tol, o.maxit, o.krylov, &its, &rr, st, true))
      return -1;
    s->iterations = its;
    s->relres = rr;
    return 0;
  }
  if (!o.fp32_inner) {
    int its;
    double rr;
    if (S.nseg > 1 ? gmres_seg<double>(C, R, dx, o.tol, o.maxit, o.krylov, &its, &rr, st)
                   : gmres<double>(C, R, dx, o.tol, o.maxit, o.krylov, &its, &rr, st))
      return -1;
    s->iterations = its;
    s->relres = rr;
    return 0;
  }
  // iterative refinement: dx = 0, r = R
  const int lpr = lanes_per_row(C->L);
  GB_CU(cudaMemsetAsync(dx, 0, sizeof(double) * N, st), "dx0");
  GB_CU(cudaMemcpyAsync(S.d_r, R, sizeof(double) * N, cudaMemcpyDeviceToDevice, st), "r0");
  double n3[3];
  if (device_norms(C, R, N, n3, st)) return -1;
  const double bnorm = n3[0];
  s->relres = 0.0;
  if (bnorm == 0.0) return 0;
  double rn = bnorm;
  // scratch: d_xs (N doubles) holds the FP32 right-hand side and solution
  float *r32 = (float *)S.d_xs;
  for (int it = 0; it < o.max_refinements; it++) {
    to_f32_scaled_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(N, S.d_r, rn, r32);
    int its;
    double rr;
    float *sol32 = (float *)S.d_xs + N;
    // each inner solve goes no further than the outer target needs (a loose
    // forcing-rule tolerance is met by one inner solve), nor further than
    // inner_tol (beyond it FP32 arithmetic limits what a solve attains)
    const double itol = std::max(o.inner_tol, o.tol * bnorm / rn);
    if (S.nseg > 1 ? gmres_seg<float>(C, r32, sol32, itol, o.maxit, o.krylov, &its, &rr, st)
                   : gmres<float>(C, r32, sol32, itol, o.maxit, o.krylov, &its, &rr, st))
      return -1;
    s->iterations += its;
    s->refinements++;
    axpy_f32_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(N, rn, sol32, dx);
    // r = R - A dx (FP64)
    GB_CU(spmv<double>(C, lpr, S.d_A, dx, S.d_r, st), "spmv64");
    residual_kernel<<<kRedBlocks, kRedThreads, 0, st>>>(N, R, S.d_r);
    if (device_norms(C, S.d_r, N, n3, st)) return -1;
    rn = n3[0];
    s->relres = rn / bnorm;
    if (rn <= o.tol * bnorm) break;
  }
  return 0;
}

}  // namespace gb
