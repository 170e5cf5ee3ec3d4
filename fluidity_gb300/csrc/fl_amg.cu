// fl_amg.cu -- smoothed-aggregation algebraic multigrid preconditioner for
// the CG solve of the pressure (Poisson) systems.
//
// The stronger preconditioner of petsc_solve's options (femtools/Solvers.F90:
// 1827-1969, PCGAMG), restated on the GPU with the structure of PETSc's GAMG
// defaults:
//   * aggregation by a distance-2 maximal independent set of the matrix graph
//     (Luby's algorithm with hashed priorities, Bell, Dalton and Olson 2012),
//     rows without off-diagonal couplings (Dirichlet ghost rows) left out;
//   * one Jacobi smoothing step of the piecewise-constant prolongator,
//     P = (I - omega D^-1 A) P0, omega = 4 / (3 rho), rho a Gershgorin bound
//     on the spectrum of D^-1 A;
//   * Galerkin coarse operators A_c = P^T A P;
//   * Chebyshev(2)-Jacobi smoothing on [0.1 rho, 1.1 rho] before and after the
//     coarse correction (a symmetric V-cycle), and a dense direct solve on the
//     coarsest level.
// Every sparse product sums its terms in a fixed order (candidates sorted by
// column and then by their position), so the hierarchy and the solve are
// deterministic.  The solve is PCG with PETSc's default convergence test on
// the preconditioned residual norm, petsc_solve's ghost semantics and rhs
// lifting, as the Jacobi solve of fl_krylov.cu.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "fl_internal.cuh"
#include "fl_device.cuh"

namespace fl {

unsigned long long launches_amg() { return unit_launches(); }

namespace {

constexpr int kT = 256;
constexpr int kCap = 8192;         // candidate entries of one row of a sparse product
constexpr int kMaxCoarse = 512;    // rows of the coarsest level (dense inverse)
constexpr int kMaxLevels = 12;

struct Csr {
  int32_t n = 0, m = 0;  // rows, columns
  int64_t nnz = 0;
  DevBuf<int32_t> ptr, col;
  DevBuf<double> val;
};

// ------------------------------------------------------------ helpers --
__device__ __forceinline__ uint32_t hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

template <int NT>
__device__ double block_sum_d(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  v = 0.0;
  if (w == 0) {
    v = lane < NT / 32 ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;
}

// y = A x for one row by G lanes (rows sorted; terms in pattern order per lane)
template <int G>
__device__ __forceinline__ double csr_row(const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                                          const double* __restrict__ val, const double* __restrict__ x, int row,
                                          int sub, bool valid) {
  int b = 0, e = 0;
  if (valid) {
    b = __ldg(ptr + row);
    e = __ldg(ptr + row + 1);
  }
  double s = 0.0;
  for (int k = b + sub; k < e; k += G) s += __ldg(val + k) * __ldg(x + __ldg(col + k));
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
  return s;
}

// ------------------------------------------------------ level-0 matrix --
// min / max of |a_ii| over every row (ghost pivot, Petsc_Tools.F90:972-983),
// as ordered bits of non-negative doubles
__global__ void k_diag_range(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                             const double* __restrict__ val, unsigned long long* mm) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k)
      if (col[k] == i) d = fabs(val[k]);
    const unsigned long long b = (unsigned long long)__double_as_longlong(d);
    atomicMin(mm, b);
    atomicMax(mm + 1, b);
  }
}

// The matrix PETSc is given: ghost rows hold only the ghost pivot on the
// diagonal, ghost columns are dropped (zero) in active rows.
__global__ void k_mask(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                       const double* __restrict__ val, const uint8_t* __restrict__ ghost,
                       const unsigned long long* __restrict__ mm, double* __restrict__ out) {
  note_launch();
  const double mind = __longlong_as_double((long long)mm[0]), maxd = __longlong_as_double((long long)mm[1]);
  const double piv = sqrt((maxd + mind) * maxd / 2.0);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const bool gi = ghost && ghost[i];
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int j = col[k];
      double v;
      if (gi) v = j == i ? piv : 0.0;
      else v = (ghost && ghost[j]) ? 0.0 : val[k];
      out[k] = v;
    }
  }
}

// 1/a_ii (0 when the row has no diagonal) and the Gershgorin bound of the
// row of D^-1 A: sum_j |a_ij| / |a_ii|
__global__ void k_dinv_gersh(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                             const double* __restrict__ val, double* __restrict__ dinv,
                             unsigned long long* __restrict__ gmax) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double d = 0.0, s = 0.0;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
      s += fabs(val[k]);
      if (col[k] == i) d = val[k];
    }
    dinv[i] = d != 0.0 ? 1.0 / d : 0.0;
    const double g = d != 0.0 ? s / fabs(d) : 0.0;
    atomicMax(gmax, (unsigned long long)__double_as_longlong(g));
  }
}

// ------------------------------------------------------- aggregation --
// tuple = state (2 bits: 2 in the set, 1 undecided, 0 out) | hash (30) | index
__device__ __forceinline__ unsigned long long tup(uint32_t st, uint32_t h, uint32_t i) {
  return ((unsigned long long)st << 62) | ((unsigned long long)(h & 0x3fffffffu) << 32) | i;
}

__device__ __forceinline__ bool coupled(const double* __restrict__ val, int k) { return val[k] != 0.0; }

__global__ void k_mis_init(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                           const double* __restrict__ val, uint32_t seed, unsigned long long* __restrict__ t,
                           int32_t* __restrict__ agg) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    bool any = false;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) any = any || (col[k] != i && coupled(val, k));
    t[i] = tup(any ? 1u : 0u, hash32((uint32_t)i * 2654435761u + seed), (uint32_t)i);
    agg[i] = -1;
  }
}

// tout_i = max of tin over i and its coupled neighbours
__global__ void k_mis_max(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                          const double* __restrict__ val, const unsigned long long* __restrict__ tin,
                          unsigned long long* __restrict__ tout) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    unsigned long long m = tin[i];
    for (int k = ptr[i]; k < ptr[i + 1]; ++k)
      if (col[k] != i && coupled(val, k)) m = max(m, tin[col[k]]);
    tout[i] = m;
  }
}

__global__ void k_mis_update(int n, unsigned long long* __restrict__ t, const unsigned long long* __restrict__ t2,
                             int* __restrict__ left) {
  note_launch();
  int c = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned long long v = t[i];
    if ((v >> 62) != 1ull) continue;
    if (t2[i] == v) t[i] = (v & ~(3ull << 62)) | (2ull << 62);  // into the set
    else if ((t2[i] >> 62) == 2ull) t[i] = v & ~(3ull << 62);   // within distance 2 of the set
    else ++c;
  }
  if (c) atomicAdd(left, c);
}

__global__ void k_mis_flag(int n, const unsigned long long* __restrict__ t, int32_t* __restrict__ flag) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    flag[i] = (t[i] >> 62) == 2ull ? 1 : 0;
}

// distance 1: the highest set member among i and its neighbours
__global__ void k_agg1(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                       const double* __restrict__ val, const unsigned long long* __restrict__ t,
                       const int32_t* __restrict__ rank, int32_t* __restrict__ agg,
                       unsigned long long* __restrict__ pick) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    unsigned long long best = (t[i] >> 62) == 2ull ? t[i] : 0ull;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int j = col[k];
      if (j != i && coupled(val, k) && (t[j] >> 62) == 2ull) best = max(best, t[j]);
    }
    pick[i] = best;
    if (best) agg[i] = rank[(uint32_t)best];
  }
}

// distance 2: the highest pick among the neighbours
__global__ void k_agg2(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                       const double* __restrict__ val, const unsigned long long* __restrict__ pick,
                       const int32_t* __restrict__ rank, int32_t* __restrict__ agg, ErrWord* err) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (agg[i] >= 0) continue;
    bool any = false;
    unsigned long long best = 0ull;
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int j = col[k];
      if (j != i && coupled(val, k)) {
        any = true;
        best = max(best, pick[j]);
      }
    }
    if (!any) continue;  // uncoupled row: no aggregate
    if (!best) {
      set_err(err, FL_ERR_UNSUPPORTED, i);  // not reachable after a maximal set
      continue;
    }
    agg[i] = rank[(uint32_t)best];
  }
}

// P0: one entry (agg(i), 1) per aggregated row
__global__ void k_p0_count(int n, const int32_t* __restrict__ agg, int32_t* __restrict__ cnt) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) cnt[i] = agg[i] >= 0;
}
__global__ void k_p0_fill(int n, const int32_t* __restrict__ agg, const int32_t* __restrict__ ptr,
                          int32_t* __restrict__ col, double* __restrict__ val) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (agg[i] >= 0) {
      col[ptr[i]] = agg[i];
      val[ptr[i]] = 1.0;
    }
}

// ------------------------------------------- deterministic sparse product --
// Row i of C = L B: candidates (col_B(q), l_ik b_kq) for k in row i of L and q
// in row k of B, sorted by (column, candidate position), summed per column in
// that order.  One block per row; pass 0 counts the columns, pass 1 fills.
struct ProdArgs {
  int32_t n;
  const int32_t* rows;  // rows to process (null: all n rows)
  const int32_t *lp, *lc;
  const double* lv;
  const int32_t *bp, *bc;
  const double* bv;
  int32_t* cnt;       // pass 0
  const int32_t* cp;  // pass 1
  int32_t* cc;
  double* cv;
  ErrWord* err;
};

template <int NT>
__global__ void __launch_bounds__(NT) k_spgemm(ProdArgs A, int pass) {
  note_launch();
  extern __shared__ unsigned char sm[];
  unsigned long long* key = reinterpret_cast<unsigned long long*>(sm);  // [kCap]
  double* v = reinterpret_cast<double*>(key + kCap);                     // [kCap]
  __shared__ int s_n, s_tot;
  __shared__ int s_scan[NT];
  for (int it = blockIdx.x; it < A.n; it += gridDim.x) {
    const int row = A.rows ? A.rows[it] : it;
    // candidate offsets: lane-parallel prefix over the row of L
    const int lb = A.lp[row], le = A.lp[row + 1];
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    for (int k0 = lb; k0 < le; k0 += NT) {
      const int k = k0 + threadIdx.x;
      const int len = k < le ? A.bp[A.lc[k] + 1] - A.bp[A.lc[k]] : 0;
      s_scan[threadIdx.x] = len;
      __syncthreads();
      for (int o = 1; o < NT; o <<= 1) {
        const int x = threadIdx.x >= o ? s_scan[threadIdx.x - o] : 0;
        __syncthreads();
        s_scan[threadIdx.x] += x;
        __syncthreads();
      }
      const int base = s_n, excl = s_scan[threadIdx.x] - len;
      if (k < le) {
        const int kk = A.lc[k];
        const double l = A.lv[k];
        const int qb = A.bp[kk];
        for (int q = 0; q < len; ++q) {
          const int pos = base + excl + q;
          if (pos < kCap) {
            key[pos] = ((unsigned long long)(uint32_t)A.bc[qb + q] << 32) | (uint32_t)pos;
            v[pos] = l * A.bv[qb + q];
          }
        }
      }
      __syncthreads();
      if (threadIdx.x == NT - 1) s_n = base + s_scan[NT - 1];
      __syncthreads();
    }
    const int nc = s_n;
    if (nc > kCap) {  // left to k_spgemm_long
      if (pass == 0 && threadIdx.x == 0) A.cnt[row] = -1;
      __syncthreads();
      continue;
    }
    int pw = 1;
    while (pw < nc) pw <<= 1;
    for (int k = nc + threadIdx.x; k < pw; k += NT) key[k] = ~0ull;
    __syncthreads();
    // bitonic sort of the keys
    for (int size = 2; size <= pw; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int k = threadIdx.x; k < pw; k += NT) {
          const int l = k ^ stride;
          if (l > k) {
            const unsigned long long a = key[k], b = key[l];
            const bool up = (k & size) == 0;
            if ((a > b) == up) {
              key[k] = b;
              key[l] = a;
            }
          }
        }
        __syncthreads();
      }
    // segment heads
    if (threadIdx.x == 0) s_tot = 0;
    __syncthreads();
    int mine = 0;
    for (int k = threadIdx.x; k < nc; k += NT) mine += (k == 0 || (key[k] >> 32) != (key[k - 1] >> 32));
    if (mine) atomicAdd(&s_tot, mine);
    __syncthreads();
    if (pass == 0) {
      if (threadIdx.x == 0) A.cnt[row] = s_tot;
      __syncthreads();
      continue;
    }
    // pass 1: output slot of each head = number of heads before it
    const int out0 = A.cp[row];
    for (int k0 = 0; k0 < nc; k0 += NT) {
      const int k = k0 + threadIdx.x;
      const int head = k < nc && (k == 0 || (key[k] >> 32) != (key[k - 1] >> 32));
      s_scan[threadIdx.x] = head;
      __syncthreads();
      for (int o = 1; o < NT; o <<= 1) {
        const int x = threadIdx.x >= o ? s_scan[threadIdx.x - o] : 0;
        __syncthreads();
        s_scan[threadIdx.x] += x;
        __syncthreads();
      }
      if (head) {
        const int slot = (k0 == 0 ? 0 : s_tot) + s_scan[threadIdx.x] - 1;
        const uint32_t c = (uint32_t)(key[k] >> 32);
        double sum = 0.0;
        for (int q = k; q < nc && (uint32_t)(key[q] >> 32) == c; ++q) sum += v[(uint32_t)key[q]];
        A.cc[out0 + slot] = (int32_t)c;
        A.cv[out0 + slot] = sum;
      }
      __syncthreads();
      if (threadIdx.x == NT - 1) s_tot = (k0 == 0 ? 0 : s_tot) + s_scan[NT - 1];
      __syncthreads();
    }
  }
}

// The same product, one warp per row, for rows of at most kWarpCap
// candidates (the common case on the finer levels); longer rows are marked
// with count -2 for the block kernel.  Same candidate order, same sort key,
// same sums: identical results to the block kernel.
constexpr int kWarpCap = 256;
constexpr int kWarpsW = 8;
__global__ void __launch_bounds__(kWarpsW * 32) k_spgemm_warp(ProdArgs A, int pass) {
  note_launch();
  __shared__ unsigned long long key_all[kWarpsW][kWarpCap];
  __shared__ double v_all[kWarpsW][kWarpCap];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned long long* key = key_all[w];
  double* v = v_all[w];
  const int nw = gridDim.x * kWarpsW;
  for (int row = blockIdx.x * kWarpsW + w; row < A.n; row += nw) {
    const int lb = A.lp[row], le = A.lp[row + 1];
    int total = 0;
    bool over = false;
    for (int k0 = lb; k0 < le; k0 += 32) {
      const int k = k0 + lane;
      const int len = k < le ? A.bp[A.lc[k] + 1] - A.bp[A.lc[k]] : 0;
      int incl = len;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += x;
      }
      const int excl = total + incl - len;
      const int chunk = __shfl_sync(0xffffffffu, incl, 31);
      if (total + chunk > kWarpCap) {
        over = true;
        break;
      }
      if (k < le) {
        const int kk = A.lc[k];
        const double l = A.lv[k];
        const int qb = A.bp[kk];
        for (int q = 0; q < len; ++q) {
          const int pos = excl + q;
          key[pos] = ((unsigned long long)(uint32_t)A.bc[qb + q] << 32) | (uint32_t)pos;
          v[pos] = l * A.bv[qb + q];
        }
      }
      total += chunk;
    }
    __syncwarp();
    if (over) {
      if (pass == 0 && lane == 0) A.cnt[row] = -2;
      continue;
    }
    const int nc = total;
    int pw = 1;
    while (pw < nc) pw <<= 1;
    for (int k = nc + lane; k < pw; k += 32) key[k] = ~0ull;
    __syncwarp();
    for (int size = 2; size <= pw; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int k = lane; k < pw; k += 32) {
          const int l = k ^ stride;
          if (l > k) {
            const unsigned long long a = key[k], b = key[l];
            const bool up = (k & size) == 0;
            if ((a > b) == up) {
              key[k] = b;
              key[l] = a;
            }
          }
        }
        __syncwarp();
      }
    // heads, their ranks (ballot prefix) and per-column sums in sorted order
    int base = 0;
    const int out0 = pass == 1 ? A.cp[row] : 0;
    for (int k0 = 0; k0 < nc; k0 += 32) {
      const int k = k0 + lane;
      const bool head = k < nc && (k == 0 || (key[k] >> 32) != (key[k - 1] >> 32));
      const unsigned m = __ballot_sync(0xffffffffu, head);
      if (pass == 1 && head) {
        const int slot = base + __popc(m & ((1u << lane) - 1u));
        const uint32_t c = (uint32_t)(key[k] >> 32);
        double sum = 0.0;
        for (int q = k; q < nc && (uint32_t)(key[q] >> 32) == c; ++q) sum += v[(uint32_t)key[q]];
        A.cc[out0 + slot] = (int32_t)c;
        A.cv[out0 + slot] = sum;
      }
      base += __popc(m);
    }
    if (pass == 0 && lane == 0) A.cnt[row] = base;
    __syncwarp();
  }
}

__global__ void k_rows_marked(int n, const int32_t* __restrict__ cnt, int mark, int32_t* __restrict__ list,
                              int* __restrict__ nl) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (cnt[i] == mark) list[atomicAdd(nl, 1)] = i;
}

// Rows with more candidates than one block's shared memory holds: one thread
// per row inserts the candidates, in their generation order, into a sorted
// list of distinct columns (at most kLongCols) in global scratch, adding
// values of equal columns in that order.  pass 0 writes the counts, pass 1
// the row.
constexpr int kLongCols = 4096;
__global__ void k_spgemm_long(ProdArgs A, const int32_t* __restrict__ rows, int nrows, int pass,
                              int32_t* __restrict__ scol, double* __restrict__ sval) {
  note_launch();
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nrows; t += gridDim.x * blockDim.x) {
    const int row = rows[t];
    int32_t* uc = scol + (int64_t)t * kLongCols;
    double* uv = sval + (int64_t)t * kLongCols;
    int nu = 0;
    bool over = false;
    for (int k = A.lp[row]; k < A.lp[row + 1] && !over; ++k) {
      const int kk = A.lc[k];
      const double l = A.lv[k];
      for (int q = A.bp[kk]; q < A.bp[kk + 1]; ++q) {
        const int c = A.bc[q];
        const double v = l * A.bv[q];
        int lo = 0, hi = nu;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (uc[mid] < c) lo = mid + 1;
          else hi = mid;
        }
        if (lo < nu && uc[lo] == c) {
          uv[lo] += v;
        } else {
          if (nu == kLongCols) {
            over = true;
            break;
          }
          for (int z = nu; z > lo; --z) {
            uc[z] = uc[z - 1];
            uv[z] = uv[z - 1];
          }
          uc[lo] = c;
          uv[lo] = v;
          ++nu;
        }
      }
    }
    if (over) {
      set_err(A.err, FL_ERR_UNSUPPORTED, row);
      nu = 0;
    }
    if (pass == 0) {
      A.cnt[row] = nu;
    } else {
      const int o = A.cp[row];
      for (int z = 0; z < nu; ++z) {
        A.cc[o + z] = uc[z];
        A.cv[o + z] = uv[z];
      }
    }
  }
}


// Transpose (rows of C = columns of B): slots by atomics, then each column's
// entries sorted by row (insertion sort; columns are short).
__global__ void k_t_count(int64_t nnz, const int32_t* __restrict__ col, int32_t* __restrict__ cnt) {
  note_launch();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz; k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(cnt + col[k], 1);
}
__global__ void k_t_fill(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                         const double* __restrict__ val, const int32_t* __restrict__ tp, int32_t* __restrict__ fill,
                         int32_t* __restrict__ tc, double* __restrict__ tv) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int k = ptr[i]; k < ptr[i + 1]; ++k) {
      const int j = col[k];
      const int s = tp[j] + atomicAdd(fill + j, 1);
      tc[s] = i;
      tv[s] = val[k];
    }
}
// Columns of up to kSortCap entries: one block per column, bitonic sort of
// (row, position) keys in shared memory.  Longer columns are marked (-1 in
// `longc`) for the thread-per-column insertion sort below.
constexpr int kSortCap = 2048;
__global__ void __launch_bounds__(256) k_t_sort_blk(int m, const int32_t* __restrict__ tp, int32_t* __restrict__ tc,
                                                    double* __restrict__ tv, int32_t* __restrict__ longc) {
  note_launch();
  __shared__ unsigned long long key[kSortCap];
  __shared__ double v[kSortCap];
  for (int j = blockIdx.x; j < m; j += gridDim.x) {
    const int b = tp[j], len = tp[j + 1] - b;
    longc[j] = len > kSortCap ? -1 : 0;
    if (len > kSortCap || len < 2) continue;
    int pw = 1;
    while (pw < len) pw <<= 1;
    for (int k = threadIdx.x; k < pw; k += 256) {
      if (k < len) {
        key[k] = ((unsigned long long)(uint32_t)tc[b + k] << 32) | (uint32_t)k;
        v[k] = tv[b + k];
      } else {
        key[k] = ~0ull;
      }
    }
    __syncthreads();
    for (int size = 2; size <= pw; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int k = threadIdx.x; k < pw; k += 256) {
          const int l = k ^ stride;
          if (l > k) {
            const unsigned long long x = key[k], y = key[l];
            const bool up = (k & size) == 0;
            if ((x > y) == up) {
              key[k] = y;
              key[l] = x;
            }
          }
        }
        __syncthreads();
      }
    for (int k = threadIdx.x; k < len; k += 256) {
      tc[b + k] = (int32_t)(key[k] >> 32);
      tv[b + k] = v[(uint32_t)key[k]];
    }
    __syncthreads();
  }
}

__global__ void k_t_sort(int m, const int32_t* __restrict__ tp, int32_t* __restrict__ tc, double* __restrict__ tv,
                         const int32_t* __restrict__ longc) {
  note_launch();
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < m; j += gridDim.x * blockDim.x) {
    if (longc[j] == 0) continue;
    const int b = tp[j], e = tp[j + 1];
    for (int k = b + 1; k < e; ++k) {
      const int c = tc[k];
      const double x = tv[k];
      int q = k - 1;
      while (q >= b && tc[q] > c) {
        tc[q + 1] = tc[q];
        tv[q + 1] = tv[q];
        --q;
      }
      tc[q + 1] = c;
      tv[q + 1] = x;
    }
  }
}

// P = P0 - omega D^-1 (A P0) on the pattern of A P0
__global__ void k_smooth_p(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                           double* __restrict__ val, const int32_t* __restrict__ agg,
                           const double* __restrict__ dinv, double omega) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int k = ptr[i]; k < ptr[i + 1]; ++k)
      val[k] = (col[k] == agg[i] ? 1.0 : 0.0) - omega * dinv[i] * val[k];
}

// --------------------------------------------------------- sliced ELL --
// The finest operator in slices of 32 rows, each padded to its longest row
// and stored column-major (entry j of the slice's rows contiguous), so that
// one thread per row reads coalesced values; padding has the row's own column
// and value 0.  Terms are summed in the row's CSR order.
template <class T>
struct SellOpT {
  int32_t n;
  const int32_t* sptr;
  const int32_t* col;
  const T* val;
};
typedef SellOpT<double> SellOp;

__global__ void k_sl_width(int n, const int32_t* __restrict__ ptr, int32_t* __restrict__ w) {
  note_launch();
  const int nsl = (n + 31) / 32;
  for (int sl = blockIdx.x * blockDim.x + threadIdx.x; sl < nsl; sl += gridDim.x * blockDim.x) {
    int m = 0;
    for (int r = sl * 32; r < min(n, sl * 32 + 32); ++r) m = max(m, ptr[r + 1] - ptr[r]);
    w[sl] = m * 32;
  }
}

__global__ void k_sl_fill(int n, const int32_t* __restrict__ ptr, const int32_t* __restrict__ col,
                          const double* __restrict__ val, const int32_t* __restrict__ sptr, int32_t* __restrict__ scol,
                          double* __restrict__ sval) {
  note_launch();
  const int nsl = (n + 31) / 32;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nsl * 32; r += gridDim.x * blockDim.x) {
    const int sl = r / 32, lane = r % 32;
    const int w = (sptr[sl + 1] - sptr[sl]) / 32;
    const bool real = r < n;
    const int b = real ? ptr[r] : 0, len = real ? ptr[r + 1] - b : 0;
    for (int j = 0; j < w; ++j) {
      const int64_t idx = (int64_t)sptr[sl] + (int64_t)j * 32 + lane;
      scol[idx] = j < len ? col[b + j] : (real ? r : 0);
      sval[idx] = j < len ? val[b + j] : 0.0;
    }
  }
}

template <class T>
__device__ __forceinline__ T sell_dot(const SellOpT<T>& S, const T* __restrict__ x, int r) {
  const int sl = r >> 5;
  const int b = __ldg(S.sptr + sl) + (r & 31), e = __ldg(S.sptr + sl + 1);
  T s = 0;
  for (int k = b; k < e; k += 32) s += __ldg(S.val + k) * __ldg(x + __ldg(S.col + k));
  return s;
}

// The V-cycle kernels compute in T (double, or float for the FP32 cycle);
// the finest level reads its rhs (TB) and writes its result (TO) in FP64.
// r = b - A x;  d = c1 d + c2 D^-1 r;  xo = x + d   (xo != x)
template <class T, class TB, class TO>
__global__ void k_cheb_sl(SellOpT<T> A, const T* __restrict__ dinv, const TB* __restrict__ b,
                          const T* __restrict__ x, T* __restrict__ d, T c1, T c2, TO* __restrict__ xo) {
  note_launch();
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n; row += gridDim.x * blockDim.x) {
    const T r = (T)b[row] - sell_dot(A, x, row);
    const T dn = (c1 != (T)0 ? c1 * d[row] : (T)0) + c2 * dinv[row] * r;
    d[row] = dn;
    xo[row] = (TO)(x[row] + dn);
  }
}

template <class T, class TB>
__global__ void k_resid_sl(SellOpT<T> A, const TB* __restrict__ b, const T* __restrict__ x, T* __restrict__ r) {
  note_launch();
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n; row += gridDim.x * blockDim.x)
    r[row] = (T)b[row] - sell_dot(A, x, row);
}

// ----------------------------------------------------------- V-cycle --
template <class T>
struct OpT {  // a CSR operator
  int32_t n;
  const int32_t* ptr;
  const int32_t* col;
  const T* val;
};
typedef OpT<double> Op;

template <int G, class T>
__device__ __forceinline__ T csr_rowT(const OpT<T>& A, const T* __restrict__ x, int row, int sub, bool valid) {
  int b = 0, e = 0;
  if (valid) {
    b = __ldg(A.ptr + row);
    e = __ldg(A.ptr + row + 1);
  }
  T s = 0;
  for (int k = b + sub; k < e; k += G) s += __ldg(A.val + k) * __ldg(x + __ldg(A.col + k));
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
  return s;
}

// x = d = (D^-1 b) / theta   (first Chebyshev step from a zero guess)
template <class T, class TB>
__global__ void k_cheb0(int n, const T* __restrict__ dinv, const TB* __restrict__ b, T ith, T* __restrict__ x,
                        T* __restrict__ d) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const T v = dinv[i] * (T)b[i] * ith;
    d[i] = v;
    x[i] = v;
  }
}

template <int G, class T, class TB, class TO>
__global__ void k_cheb(OpT<T> A, const T* __restrict__ dinv, const TB* __restrict__ b, const T* __restrict__ x,
                       T* __restrict__ d, T c1, T c2, TO* __restrict__ xo) {
  note_launch();
  const int lane = threadIdx.x & 31, sub = lane & (G - 1), gpb = blockDim.x / G;
  for (int base = blockIdx.x * gpb; base < A.n; base += gridDim.x * gpb) {
    const int row = base + threadIdx.x / G;
    const T ax = csr_rowT<G>(A, x, row, sub, row < A.n);
    if (row < A.n && sub == 0) {
      const T r = (T)b[row] - ax;
      const T dn = (c1 != (T)0 ? c1 * d[row] : (T)0) + c2 * dinv[row] * r;
      d[row] = dn;
      xo[row] = (TO)(x[row] + dn);
    }
  }
}

// r = b - A x (FP64; the solve's own residuals)
template <int G>
__global__ void k_resid(Op A, const double* __restrict__ b, const double* __restrict__ x, double* __restrict__ r) {
  note_launch();
  const int lane = threadIdx.x & 31, sub = lane & (G - 1), gpb = blockDim.x / G;
  for (int base = blockIdx.x * gpb; base < A.n; base += gridDim.x * gpb) {
    const int row = base + threadIdx.x / G;
    const double ax = csr_rowT<G>(A, x, row, sub, row < A.n);
    if (row < A.n && sub == 0) r[row] = b[row] - ax;
  }
}

template <int G, class T, class TB>
__global__ void k_residT(OpT<T> A, const TB* __restrict__ b, const T* __restrict__ x, T* __restrict__ r) {
  note_launch();
  const int lane = threadIdx.x & 31, sub = lane & (G - 1), gpb = blockDim.x / G;
  for (int base = blockIdx.x * gpb; base < A.n; base += gridDim.x * gpb) {
    const int row = base + threadIdx.x / G;
    const T ax = csr_rowT<G>(A, x, row, sub, row < A.n);
    if (row < A.n && sub == 0) r[row] = (T)b[row] - ax;
  }
}

// y = A x (+ z when z is not null)
template <int G, class T>
__global__ void k_spmv_add(OpT<T> A, const T* __restrict__ x, const T* z, T* y) {
  note_launch();
  const int lane = threadIdx.x & 31, sub = lane & (G - 1), gpb = blockDim.x / G;
  for (int base = blockIdx.x * gpb; base < A.n; base += gridDim.x * gpb) {
    const int row = base + threadIdx.x / G;
    const T ax = csr_rowT<G>(A, x, row, sub, row < A.n);
    if (row < A.n && sub == 0) y[row] = (z ? z[row] : (T)0) + ax;
  }
}

// coarsest level: x = Ainv b, one warp per row, terms in column order
template <class T, class TB, class TO>
__global__ void k_dense(int n, const T* __restrict__ inv, const TB* __restrict__ b, TO* __restrict__ x) {
  note_launch();
  const int lane = threadIdx.x & 31;
  for (int row = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < n; row += gridDim.x * (blockDim.x >> 5)) {
    T s = 0;
    for (int j = lane; j < n; j += 32) s += inv[(int64_t)row * n + j] * (T)b[j];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) x[row] = (TO)s;
  }
}

__global__ void k_to_float(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  note_launch();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// ------------------------------------------------------------ PCG --
struct AmgState {
  double rtol, atol, dtol, rnorm0, ttol, rnorm;
  double alpha, beta, betaold, dpi, dpiold, pcoef;
  double true_r2, b2;
  int its, max_its, reason, done, guess_zero, i;
};

__device__ void amg_converged(AmgState& S, int it, double rn, double bn) {
  if (it == 0) {
    S.rnorm0 = S.guess_zero ? rn : (bn > 0.0 ? bn : rn);
    S.ttol = fmax(S.rtol * S.rnorm0, S.atol);
  }
  S.rnorm = rn;
  if (rn != rn) S.reason = FL_DIVERGED_NANORINF;
  else if (rn <= S.ttol) S.reason = rn < S.atol ? FL_CONVERGED_ATOL : FL_CONVERGED_RTOL;
  else if (rn >= S.dtol * S.rnorm0) S.reason = FL_DIVERGED_DTOL;
  if (S.reason) S.done = 1;
}

// b = rhs - A (rhs on ghosts) on active rows, 0 on ghosts; y = guess (0 on ghosts)
template <int G>
__global__ void k_amg_lift(Op A, const uint8_t* __restrict__ ghost, const double* __restrict__ rhs,
                           const double* __restrict__ x0, int guess_zero, double* __restrict__ b,
                           double* __restrict__ y) {
  note_launch();
  const int lane = threadIdx.x & 31, sub = lane & (G - 1), gpb = blockDim.x / G;
  for (int base = blockIdx.x * gpb; base < A.n; base += gridDim.x * gpb) {
    const int row = base + threadIdx.x / G;
    double s = 0.0;
    if (row < A.n && ghost) {
      for (int k = __ldg(A.ptr + row) + sub; k < __ldg(A.ptr + row + 1); k += G) {
        const int j = A.col[k];
        if (ghost[j]) s += A.val[k] * rhs[j];
      }
    }
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
    if (row < A.n && sub == 0) {
      const bool g = ghost && ghost[row];
      b[row] = g ? 0.0 : rhs[row] - s;
      y[row] = (guess_zero || g) ? 0.0 : x0[row];
    }
  }
}

// partials of a.b and c.d over blocks (two dots in one pass; c may be null)
__global__ void k_dots(int n, const double* __restrict__ a, const double* __restrict__ b,
                       const double* __restrict__ c, const double* __restrict__ d, double* __restrict__ part) {
  note_launch();
  __shared__ double red[kT / 32];
  double s = 0.0, t = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    s += a[i] * b[i];
    if (c) t += c[i] * d[i];
  }
  s = block_sum_d<kT>(s, red);
  t = block_sum_d<kT>(t, red);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = s;
    part[gridDim.x + blockIdx.x] = t;
  }
}

// w = A p and partials of p.w
template <int G>
__global__ void k_amg_ap(Op A, const AmgState* st, const double* __restrict__ p, double* __restrict__ w,
                         double* __restrict__ part) {
  note_launch();
  __shared__ double red[kT / 32];
  if (st->done) return;
  const int lane = threadIdx.x & 31, sub = lane & (G - 1), gpb = blockDim.x / G;
  double pw = 0.0;
  for (int base = blockIdx.x * gpb; base < A.n; base += gridDim.x * gpb) {
    const int row = base + threadIdx.x / G;
    const double s = csr_row<G>(A.ptr, A.col, A.val, p, row, sub, row < A.n);
    if (row < A.n && sub == 0) {
      w[row] = s;
      pw += p[row] * s;
    }
  }
  pw = block_sum_d<kT>(pw, red);
  if (threadIdx.x == 0) part[blockIdx.x] = pw;
}

// w = A p and partials of p.w on the sliced-ELL finest operator
__global__ void k_amg_ap_sl(SellOp A, const AmgState* st, const double* __restrict__ p, double* __restrict__ w,
                            double* __restrict__ part) {
  note_launch();
  __shared__ double red[kT / 32];
  if (st->done) return;
  double pw = 0.0;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n; row += gridDim.x * blockDim.x) {
    const double s = sell_dot(A, p, row);
    w[row] = s;
    pw += p[row] * s;
  }
  pw = block_sum_d<kT>(pw, red);
  if (threadIdx.x == 0) part[blockIdx.x] = pw;
}

__device__ double sum_parts(const double* __restrict__ part, int n, double* red) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += kT) s += part[i];
  return block_sum_d<kT>(s, red);
}

// alpha = beta / p.w (KSPSolve_CG)
__global__ void k_amg_alpha(AmgState* st, const double* __restrict__ part, int nparts) {
  note_launch();
  __shared__ double red[kT / 32];
  if (st->done) return;
  const double dpi = sum_parts(part, nparts, red);
  if (threadIdx.x) return;
  AmgState& S = *st;
  S.dpiold = S.dpi;
  S.dpi = dpi;
  S.betaold = S.beta;
  if (dpi == 0.0 || (S.i > 0 && dpi * S.dpiold <= 0.0)) {
    S.reason = FL_DIVERGED_INDEFINITE_MAT;
    S.done = 1;
  } else {
    S.alpha = S.beta / dpi;
  }
}

__global__ void k_amg_xr(int n, const AmgState* st, const double* __restrict__ p, const double* __restrict__ w,
                         double* __restrict__ y, double* __restrict__ r) {
  note_launch();
  if (st->done) return;
  const double a = st->alpha;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    y[i] += a * p[i];
    r[i] -= a * w[i];
  }
}

// after z = B r: convergence test on ||z|| at iteration i+1, beta = z.r
__global__ void k_amg_beta(AmgState* st, const double* __restrict__ part, int nparts, int first,
                           const double* __restrict__ bnorm) {
  note_launch();
  __shared__ double red[kT / 32];
  if (st->done) return;
  const double zz = sum_parts(part, nparts, red);
  const double zr = sum_parts(part + nparts, nparts, red);
  if (threadIdx.x) return;
  AmgState& S = *st;
  if (first) {
    S.its = 0;
    amg_converged(S, 0, sqrt(zz), bnorm ? *bnorm : 0.0);
    S.beta = zr;
    S.pcoef = 0.0;
    S.i = 0;
    if (!S.done && zr == 0.0) {
      S.reason = FL_CONVERGED_ATOL;
      S.done = 1;
    }
    return;
  }
  const int it = S.i + 1;
  S.its = it;
  amg_converged(S, it, sqrt(zz), 0.0);
  if (S.done) return;
  if (it >= S.max_its) {
    S.reason = FL_DIVERGED_ITS;
    S.done = 1;
    return;
  }
  S.beta = zr;
  if (zr * S.betaold < 0.0) {
    S.reason = FL_DIVERGED_INDEFINITE_PC;
    S.done = 1;
    return;
  }
  S.pcoef = zr / S.betaold;
  S.i = it;
}

__global__ void k_amg_p(int n, const AmgState* st, const double* __restrict__ z, double* __restrict__ p) {
  note_launch();
  if (st->done) return;
  const double c = st->pcoef;
  const bool first = st->i == 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    p[i] = first ? z[i] : z[i] + c * p[i];
}

__global__ void k_amg_norm_b(const double* __restrict__ part, int nparts, double* out) {
  note_launch();
  __shared__ double red[kT / 32];
  const double s = sum_parts(part, nparts, red);
  if (threadIdx.x == 0) *out = sqrt(s);
}

__global__ void k_amg_true(AmgState* st, const double* __restrict__ part, int nparts) {
  note_launch();
  __shared__ double red[kT / 32];
  const double rr = sum_parts(part, nparts, red);
  const double bb = sum_parts(part + nparts, nparts, red);
  if (threadIdx.x == 0) {
    st->true_r2 = rr;
    st->b2 = bb;
  }
}

__global__ void k_amg_copy_back(int n, const uint8_t* __restrict__ ghost, const double* __restrict__ rhs,
                                const double* __restrict__ y, double* __restrict__ x) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] = (ghost && ghost[i]) ? rhs[i] : y[i];
}

// lanes per row of a CSR product: about four entries per lane, 2..32 lanes
int lanes_for(const Csr& A) {
  const double avg = A.n ? (double)A.nnz / A.n : 0.0;
  int g = 2;
  while (g < 32 && g * 4 < avg) g <<= 1;
  return g;
}

}  // namespace
}  // namespace fl

using namespace fl;

struct AmgLevel {
  Csr A, P, R;
  DevBuf<int32_t> sptr, scol;  // sliced-ELL copy of A (finest level)
  DevBuf<double> sval;
  bool sell = false;
  DevBuf<double> dinv, x0, x1, d, b, r, xc;  // xc: the V-cycle's result on this level
  // single-precision copies of the operators and work vectors (FP32 cycle)
  DevBuf<float> Af, Pf, Rf, sf, dinvf, x0f, x1f, df, bf, rf, xcf;
  double rho = 2.0;  // Gershgorin bound of the spectrum of D^-1 A
  int G = 2, GP = 2, GR = 2;  // lanes per row of A, P and R
};

struct fl_amg_t {
  fl_mesh_t* m = nullptr;
  const double* val = nullptr;    // caller's matrix (rhs lifting)
  const uint8_t* ghost = nullptr;  // caller's inactive mask
  std::vector<std::unique_ptr<AmgLevel>> L;
  int nc = 0;  // rows of the coarsest level
  DevBuf<double> cinv;
  // solve work
  DevBuf<double> bb, y, r, z, p, w, part, bnorm;
  DevBuf<AmgState> st;
  int unprec = 0;  // 1: convergence test on ||r|| (KSP_NORM_UNPRECONDITIONED)
  int fp32 = 0;    // 1: the V-cycle runs in FP32 (operators and vectors)
  DevBuf<float> cinvf;
  cudaStream_t cs = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  ~fl_amg_t() {
    if (cs) cudaStreamDestroy(cs);
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
  }
};

namespace {

int spgemm(const Csr& Lm, const Csr& B, Csr& C, ErrWord* err, cudaStream_t s) {
  // rows go to the warp kernel (up to kWarpCap candidates), the block kernel
  // (up to kCap) or the one-thread-per-row kernel (longer)
  C.n = Lm.n;
  C.m = B.m;
  DevBuf<int32_t> cnt, list2, list1;
  DevBuf<int> nl;
  FL_TRY(cnt.reserve((size_t)Lm.n + 1));
  FL_TRY(C.ptr.reserve((size_t)Lm.n + 1));
  FL_TRY(list2.reserve((size_t)Lm.n));
  FL_TRY(list1.reserve((size_t)Lm.n));
  FL_TRY(nl.reserve(2));
  ProdArgs A{Lm.n, nullptr, Lm.ptr.p, Lm.col.p, Lm.val.p, B.ptr.p, B.col.p, B.val.p, cnt.p, nullptr, nullptr,
             nullptr, err};
  const size_t smem = (size_t)kCap * (sizeof(unsigned long long) + sizeof(double));
  static bool configured = false;
  if (!configured) {
    FL_TRY_CUDA(cudaFuncSetAttribute(k_spgemm<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured = true;
  }
  const unsigned gw = (unsigned)std::max(1, std::min((Lm.n + kWarpsW - 1) / kWarpsW, num_sms() * 8));
  k_spgemm_warp<<<gw, kWarpsW * 32, 0, s>>>(A, 0);
  FL_TRY_CUDA(cudaMemsetAsync(nl.p, 0, sizeof(int) * 2, s));
  k_rows_marked<<<grid_for(Lm.n, kT), kT, 0, s>>>(Lm.n, cnt.p, -2, list2.p, nl.p);
  int hn[2] = {0, 0};
  FL_TRY_CUDA(cudaMemcpyAsync(hn, nl.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  const int nblock = hn[0];
  ProdArgs Ab = A;
  Ab.n = nblock;
  Ab.rows = list2.p;
  const unsigned gb = (unsigned)std::max(1, std::min(nblock, num_sms() * 8));
  int nlong = 0;
  if (nblock > 0) {
    k_spgemm<256><<<gb, 256, smem, s>>>(Ab, 0);
    k_rows_marked<<<grid_for(Lm.n, kT), kT, 0, s>>>(Lm.n, cnt.p, -1, list1.p, nl.p + 1);
    FL_TRY_CUDA(cudaMemcpyAsync(&nlong, nl.p + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    FL_TRY_CUDA(cudaStreamSynchronize(s));
  }
  DevBuf<int32_t> lcol;
  DevBuf<double> lval;
  if (nlong > 0) {
    if (nlong > (1 << 16)) {
      set_error("sparse product: %d rows above the candidate capacity", nlong);
      return FL_ERR_UNSUPPORTED;
    }
    FL_TRY(lcol.reserve((size_t)nlong * kLongCols));
    FL_TRY(lval.reserve((size_t)nlong * kLongCols));
    k_spgemm_long<<<grid_for(nlong, 64), 64, 0, s>>>(A, list1.p, nlong, 0, lcol.p, lval.p);
  }
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY(check_err(err, s, "sparse product row with more distinct columns than the scratch holds"));
  FL_TRY(exclusive_scan_i32(cnt.p, C.ptr.p, Lm.n, s));
  int32_t nnz = 0;
  FL_TRY_CUDA(cudaMemcpyAsync(&nnz, C.ptr.p + Lm.n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  C.nnz = nnz;
  FL_TRY(C.col.reserve((size_t)std::max(nnz, 1)));
  FL_TRY(C.val.reserve((size_t)std::max(nnz, 1)));
  A.cp = Ab.cp = C.ptr.p;
  A.cc = Ab.cc = C.col.p;
  A.cv = Ab.cv = C.val.p;
  k_spgemm_warp<<<gw, kWarpsW * 32, 0, s>>>(A, 1);
  if (nblock > 0) k_spgemm<256><<<gb, 256, smem, s>>>(Ab, 1);
  if (nlong > 0) k_spgemm_long<<<grid_for(nlong, 64), 64, 0, s>>>(A, list1.p, nlong, 1, lcol.p, lval.p);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY_CUDA(cudaStreamSynchronize(s));  // scratch buffers are released on return
  return FL_OK;
}

int transpose(const Csr& B, Csr& T, cudaStream_t s) {
  T.n = B.m;
  T.m = B.n;
  T.nnz = B.nnz;
  DevBuf<int32_t> cnt, fill;
  FL_TRY(cnt.reserve((size_t)B.m + 1));
  FL_TRY(fill.reserve((size_t)B.m + 1));
  FL_TRY(T.ptr.reserve((size_t)B.m + 1));
  FL_TRY(T.col.reserve((size_t)std::max<int64_t>(B.nnz, 1)));
  FL_TRY(T.val.reserve((size_t)std::max<int64_t>(B.nnz, 1)));
  FL_TRY_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (B.m + 1), s));
  FL_TRY_CUDA(cudaMemsetAsync(fill.p, 0, sizeof(int32_t) * (B.m + 1), s));
  k_t_count<<<grid_for(B.nnz, kT), kT, 0, s>>>(B.nnz, B.col.p, cnt.p);
  FL_TRY(exclusive_scan_i32(cnt.p, T.ptr.p, B.m, s));
  k_t_fill<<<grid_for(B.n, kT), kT, 0, s>>>(B.n, B.ptr.p, B.col.p, B.val.p, T.ptr.p, fill.p, T.col.p, T.val.p);
  DevBuf<int32_t> longc;
  FL_TRY(longc.reserve((size_t)B.m + 1));
  k_t_sort_blk<<<(unsigned)std::max(1, std::min(B.m, num_sms() * 8)), 256, 0, s>>>(B.m, T.ptr.p, T.col.p, T.val.p,
                                                                                   longc.p);
  k_t_sort<<<grid_for(B.m, kT), kT, 0, s>>>(B.m, T.ptr.p, T.col.p, T.val.p, longc.p);
  FL_TRY_CUDA(cudaStreamSynchronize(s));  // longc is released on return
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

// Dense inverse of a small SPD matrix by Cholesky (host, once per hierarchy).
int dense_inverse(const std::vector<double>& a, int n, std::vector<double>& inv) {
  std::vector<double> l(a);
  for (int j = 0; j < n; ++j) {
    double d = l[(size_t)j * n + j];
    for (int k = 0; k < j; ++k) d -= l[(size_t)j * n + k] * l[(size_t)j * n + k];
    if (!(d > 0.0)) {
      set_error("coarsest AMG operator is not positive definite");
      return FL_ERR_UNSUPPORTED;
    }
    d = std::sqrt(d);
    l[(size_t)j * n + j] = d;
    for (int i = j + 1; i < n; ++i) {
      double s = l[(size_t)i * n + j];
      for (int k = 0; k < j; ++k) s -= l[(size_t)i * n + k] * l[(size_t)j * n + k];
      l[(size_t)i * n + j] = s / d;
    }
  }
  inv.assign((size_t)n * n, 0.0);
  std::vector<double> y(n);
  for (int c = 0; c < n; ++c) {
    for (int i = 0; i < n; ++i) {  // L y = e_c
      double s = i == c ? 1.0 : 0.0;
      for (int k = 0; k < i; ++k) s -= l[(size_t)i * n + k] * y[k];
      y[i] = s / l[(size_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; --i) {  // L^T x = y
      double s = y[i];
      for (int k = i + 1; k < n; ++k) s -= l[(size_t)k * n + i] * inv[(size_t)k * n + c];
      inv[(size_t)i * n + c] = s / l[(size_t)i * n + i];
    }
  }
  return FL_OK;
}

int level_setup(AmgLevel& Lv, cudaStream_t s) {
  const int n = Lv.A.n;
  FL_TRY(Lv.dinv.reserve(n));
  DevBuf<unsigned long long> g;
  FL_TRY(g.reserve(1));
  FL_TRY_CUDA(cudaMemsetAsync(g.p, 0, sizeof(unsigned long long), s));
  k_dinv_gersh<<<grid_for(n, kT), kT, 0, s>>>(n, Lv.A.ptr.p, Lv.A.col.p, Lv.A.val.p, Lv.dinv.p, g.p);
  unsigned long long hb = 0;
  FL_TRY_CUDA(cudaMemcpyAsync(&hb, g.p, sizeof(hb), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  double rho;
  std::memcpy(&rho, &hb, sizeof(rho));
  Lv.rho = rho > 0.0 ? rho : 1.0;
  Lv.G = lanes_for(Lv.A);
  FL_TRY(Lv.x0.reserve(n));
  FL_TRY(Lv.x1.reserve(n));
  FL_TRY(Lv.d.reserve(n));
  FL_TRY(Lv.b.reserve(n));
  FL_TRY(Lv.r.reserve(n));
  FL_TRY(Lv.xc.reserve(n));
  return FL_OK;
}

// Aggregates of level Lv and its prolongator; returns the coarse size.
int coarsen(AmgLevel& Lv, int level, ErrWord* err, cudaStream_t s, int* nc_out) {
  const int n = Lv.A.n;
  const Csr& A = Lv.A;
  DevBuf<unsigned long long> t, t1, t2, pick;
  DevBuf<int32_t> agg, flag, rank;
  DevBuf<int> left;
  FL_TRY(t.reserve(n));
  FL_TRY(t1.reserve(n));
  FL_TRY(t2.reserve(n));
  FL_TRY(pick.reserve(n));
  FL_TRY(agg.reserve(n));
  FL_TRY(flag.reserve(n));
  FL_TRY(rank.reserve((size_t)n + 1));
  FL_TRY(left.reserve(1));
  const unsigned gr = grid_for(n, kT);
  k_mis_init<<<gr, kT, 0, s>>>(n, A.ptr.p, A.col.p, A.val.p, 0x9e3779b9u * (uint32_t)(level + 1), t.p, agg.p);
  for (int round = 0; round < 200; ++round) {
    k_mis_max<<<gr, kT, 0, s>>>(n, A.ptr.p, A.col.p, A.val.p, t.p, t1.p);
    k_mis_max<<<gr, kT, 0, s>>>(n, A.ptr.p, A.col.p, A.val.p, t1.p, t2.p);
    FL_TRY_CUDA(cudaMemsetAsync(left.p, 0, sizeof(int), s));
    k_mis_update<<<gr, kT, 0, s>>>(n, t.p, t2.p, left.p);
    int h = 0;
    FL_TRY_CUDA(cudaMemcpyAsync(&h, left.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    FL_TRY_CUDA(cudaStreamSynchronize(s));
    if (h == 0) break;
    if (round == 199) {
      set_error("aggregation did not converge");
      return FL_ERR_UNSUPPORTED;
    }
  }
  k_mis_flag<<<gr, kT, 0, s>>>(n, t.p, flag.p);
  FL_TRY(exclusive_scan_i32(flag.p, rank.p, n, s));
  int32_t nc = 0;
  FL_TRY_CUDA(cudaMemcpyAsync(&nc, rank.p + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  *nc_out = nc;
  if (nc == 0) return FL_OK;
  k_agg1<<<gr, kT, 0, s>>>(n, A.ptr.p, A.col.p, A.val.p, t.p, rank.p, agg.p, pick.p);
  k_agg2<<<gr, kT, 0, s>>>(n, A.ptr.p, A.col.p, A.val.p, pick.p, rank.p, agg.p, err);
  FL_TRY(check_err(err, s, "aggregation left a coupled row without an aggregate"));
  // P0 and the smoothed prolongator
  Csr P0;
  P0.n = n;
  P0.m = nc;
  FL_TRY(P0.ptr.reserve((size_t)n + 1));
  k_p0_count<<<gr, kT, 0, s>>>(n, agg.p, flag.p);
  FL_TRY(exclusive_scan_i32(flag.p, P0.ptr.p, n, s));
  int32_t nnz0 = 0;
  FL_TRY_CUDA(cudaMemcpyAsync(&nnz0, P0.ptr.p + n, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  P0.nnz = nnz0;
  FL_TRY(P0.col.reserve((size_t)std::max(nnz0, 1)));
  FL_TRY(P0.val.reserve((size_t)std::max(nnz0, 1)));
  k_p0_fill<<<gr, kT, 0, s>>>(n, agg.p, P0.ptr.p, P0.col.p, P0.val.p);
  FL_TRY(spgemm(A, P0, Lv.P, err, s));  // A P0
  const double omega = 4.0 / (3.0 * Lv.rho);
  k_smooth_p<<<gr, kT, 0, s>>>(n, Lv.P.ptr.p, Lv.P.col.p, Lv.P.val.p, agg.p, Lv.dinv.p, omega);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY(transpose(Lv.P, Lv.R, s));
  Lv.GP = lanes_for(Lv.P);
  Lv.GR = lanes_for(Lv.R);
  return FL_OK;
}

// ------------------------------------------------------- V-cycle launch --
#define FL_AMG_G(G, KERNEL, GRID, S, ...)                                           \
  do {                                                                              \
    switch (G) {                                                                    \
      case 32: KERNEL<32><<<GRID, kT, 0, S>>>(__VA_ARGS__); break;                   \
      case 16: KERNEL<16><<<GRID, kT, 0, S>>>(__VA_ARGS__); break;                   \
      case 8: KERNEL<8><<<GRID, kT, 0, S>>>(__VA_ARGS__); break;                     \
      case 4: KERNEL<4><<<GRID, kT, 0, S>>>(__VA_ARGS__); break;                     \
      default: KERNEL<2><<<GRID, kT, 0, S>>>(__VA_ARGS__); break;                    \
    }                                                                               \
  } while (0)

Op op_of(const Csr& A) { return Op{A.n, A.ptr.p, A.col.p, A.val.p}; }

// Chebyshev(2) coefficients on [0.1 rho, 1.1 rho]
struct Cheb {
  double ith, c1, c2;
};
Cheb cheb_of(double rho) {
  const double lo = 0.1 * rho, hi = 1.1 * rho;
  const double th = 0.5 * (hi + lo), de = 0.5 * (hi - lo), sg = th / de;
  const double r0 = 1.0 / sg, r1 = 1.0 / (2.0 * sg - r0);
  return Cheb{1.0 / th, r1 * r0, 2.0 * r1 / de};
}

// the operators and vectors of a level in the cycle's precision
template <class T>
struct View {
  const T *Av, *Pv, *Rv, *sv, *dinv;
  T *x0, *x1, *d, *b, *r, *xc;
};
View<double> view(AmgLevel& L, double*) {
  return View<double>{L.A.val.p, L.P.val.p, L.R.val.p, L.sval.p, L.dinv.p,
                      L.x0.p,    L.x1.p,    L.d.p,     L.b.p,    L.r.p,    L.xc.p};
}
View<float> view(AmgLevel& L, float*) {
  return View<float>{L.Af.p, L.Pf.p, L.Rf.p, L.sf.p, L.dinvf.p, L.x0f.p, L.x1f.p, L.df.p, L.bf.p, L.rf.p, L.xcf.p};
}

#define FL_AMG_SWITCH(G, CALL)            \
  switch (G) {                            \
    case 32: { constexpr int GG = 32; CALL; } break; \
    case 16: { constexpr int GG = 16; CALL; } break; \
    case 8: { constexpr int GG = 8; CALL; } break;   \
    case 4: { constexpr int GG = 4; CALL; } break;   \
    default: { constexpr int GG = 2; CALL; } break;  \
  }

// x_l = V(b_l), all on stream s (capturable); T the arithmetic of the cycle,
// TB / TO the types of its rhs and result (FP64 on the finest level)
template <class T, class TB, class TO>
void vcycle(fl_amg_t* H, int l, const TB* b, TO* x, cudaStream_t s) {
  if (l == (int)H->L.size() - 1) {
    const T* inv = nullptr;
    if constexpr (sizeof(T) == 8) inv = reinterpret_cast<const T*>(H->cinv.p);
    else inv = reinterpret_cast<const T*>(H->cinvf.p);
    k_dense<T, TB, TO><<<grid_for((int64_t)H->nc * 32, kT, 4), kT, 0, s>>>(H->nc, inv, b, x);
    return;
  }
  AmgLevel& Lv = *H->L[l];
  AmgLevel& Ln = *H->L[l + 1];
  const View<T> V = view(Lv, (T*)nullptr), W = view(Ln, (T*)nullptr);
  const int n = Lv.A.n, G = Lv.G;
  const OpT<T> A{n, Lv.A.ptr.p, Lv.A.col.p, V.Av};
  const SellOpT<T> S{n, Lv.sptr.p, Lv.scol.p, V.sv};
  const Cheb c = cheb_of(Lv.rho);
  const T ith = (T)c.ith, c1 = (T)c.c1, c2 = (T)c.c2;
  const unsigned gv = grid_for(n, kT, 4), gs = grid_for((int64_t)n * G, kT, 8), gl = grid_for(n, kT, 8);
  // pre-smoothing from zero: two Chebyshev steps (one product)
  k_cheb0<T, TB><<<gv, kT, 0, s>>>(n, V.dinv, b, ith, V.x0, V.d);
  if (Lv.sell) k_cheb_sl<T, TB, T><<<gl, kT, 0, s>>>(S, V.dinv, b, V.x0, V.d, c1, c2, V.x1);
  else FL_AMG_SWITCH(G, (k_cheb<GG, T, TB, T><<<gs, kT, 0, s>>>(A, V.dinv, b, V.x0, V.d, c1, c2, V.x1)));
  // restriction of the residual, coarse correction, prolongation
  if (Lv.sell) k_resid_sl<T, TB><<<gl, kT, 0, s>>>(S, b, V.x1, V.r);
  else FL_AMG_SWITCH(G, (k_residT<GG, T, TB><<<gs, kT, 0, s>>>(A, b, V.x1, V.r)));
  const OpT<T> R{Ln.A.n, Lv.R.ptr.p, Lv.R.col.p, V.Rv};
  const OpT<T> P{n, Lv.P.ptr.p, Lv.P.col.p, V.Pv};
  const unsigned gr = grid_for((int64_t)Ln.A.n * Lv.GR, kT, 8), gp = grid_for((int64_t)n * Lv.GP, kT, 8);
  FL_AMG_SWITCH(Lv.GR, (k_spmv_add<GG, T><<<gr, kT, 0, s>>>(R, V.r, (const T*)nullptr, W.b)));
  vcycle<T, T, T>(H, l + 1, W.b, W.xc, s);
  FL_AMG_SWITCH(Lv.GP, (k_spmv_add<GG, T><<<gp, kT, 0, s>>>(P, W.xc, V.x1, V.x0)));
  // post-smoothing: two Chebyshev steps from the corrected guess
  if (Lv.sell) {
    k_cheb_sl<T, TB, T><<<gl, kT, 0, s>>>(S, V.dinv, b, V.x0, V.d, (T)0, ith, V.x1);
    k_cheb_sl<T, TB, TO><<<gl, kT, 0, s>>>(S, V.dinv, b, V.x1, V.d, c1, c2, x);
  } else {
    FL_AMG_SWITCH(G, (k_cheb<GG, T, TB, T><<<gs, kT, 0, s>>>(A, V.dinv, b, V.x0, V.d, (T)0, ith, V.x1)));
    FL_AMG_SWITCH(G, (k_cheb<GG, T, TB, TO><<<gs, kT, 0, s>>>(A, V.dinv, b, V.x1, V.d, c1, c2, x)));
  }
}

// the preconditioner z = B r in the handle's precision
void precondition(fl_amg_t* H, const double* r, double* z, cudaStream_t s) {
  if (H->fp32) vcycle<float, double, double>(H, 0, r, z, s);
  else vcycle<double, double, double>(H, 0, r, z, s);
}

// single-precision copies of every level's operators and vectors
int make_fp32(fl_amg_t* H, cudaStream_t s) {
  auto conv = [&](const double* a, DevBuf<float>& b, int64_t n) -> int {
    FL_TRY(b.reserve((size_t)std::max<int64_t>(n, 1)));
    if (n > 0) k_to_float<<<grid_for(n, kT), kT, 0, s>>>(n, a, b.p);
    return FL_OK;
  };
  for (size_t l = 0; l < H->L.size(); ++l) {
    AmgLevel& L = *H->L[l];
    const int n = L.A.n;
    FL_TRY(conv(L.A.val.p, L.Af, L.A.nnz));
    FL_TRY(conv(L.dinv.p, L.dinvf, n));
    if (L.sell) FL_TRY(conv(L.sval.p, L.sf, (int64_t)L.sval.n));
    if (l + 1 < H->L.size()) {
      FL_TRY(conv(L.P.val.p, L.Pf, L.P.nnz));
      FL_TRY(conv(L.R.val.p, L.Rf, L.R.nnz));
    }
    FL_TRY(L.x0f.reserve(n));
    FL_TRY(L.x1f.reserve(n));
    FL_TRY(L.df.reserve(n));
    FL_TRY(L.bf.reserve(n));
    FL_TRY(L.rf.reserve(n));
    FL_TRY(L.xcf.reserve(n));
  }
  FL_TRY(conv(H->cinv.p, H->cinvf, (int64_t)H->nc * H->nc));
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  return FL_OK;
}

}  // namespace

namespace {

int make_sell(AmgLevel& Lv, cudaStream_t s) {
  const int n = Lv.A.n, nsl = (n + 31) / 32;
  DevBuf<int32_t> w;
  FL_TRY(w.reserve((size_t)nsl + 1));
  FL_TRY(Lv.sptr.reserve((size_t)nsl + 1));
  k_sl_width<<<grid_for(nsl, kT), kT, 0, s>>>(n, Lv.A.ptr.p, w.p);
  FL_TRY(exclusive_scan_i32(w.p, Lv.sptr.p, nsl, s));
  int32_t len = 0;
  FL_TRY_CUDA(cudaMemcpyAsync(&len, Lv.sptr.p + nsl, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  FL_TRY(Lv.scol.reserve((size_t)len));
  FL_TRY(Lv.sval.reserve((size_t)len));
  k_sl_fill<<<grid_for((int64_t)nsl * 32, kT), kT, 0, s>>>(n, Lv.A.ptr.p, Lv.A.col.p, Lv.A.val.p, Lv.sptr.p,
                                                           Lv.scol.p, Lv.sval.p);
  FL_TRY_CUDA(cudaGetLastError());
  Lv.sell = true;
  return FL_OK;
}

int build_hierarchy(fl_amg_t* H, cudaStream_t s) {
  fl_mesh_t* m = H->m;
  const int n = m->N;
  DevBuf<ErrWord> err;
  FL_TRY(err.reserve(1));
  FL_TRY_CUDA(cudaMemsetAsync(err.p, 0, sizeof(ErrWord), s));
  // level 0: the ghost-masked matrix on the mesh pattern
  H->L.emplace_back(new AmgLevel());
  AmgLevel& L0 = *H->L[0];
  L0.A.n = L0.A.m = n;
  L0.A.nnz = m->nnz;
  FL_TRY(L0.A.ptr.reserve((size_t)n + 1));
  FL_TRY(L0.A.col.reserve((size_t)m->nnz));
  FL_TRY(L0.A.val.reserve((size_t)m->nnz));
  FL_TRY_CUDA(cudaMemcpyAsync(L0.A.ptr.p, m->findrm.p, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToDevice, s));
  FL_TRY_CUDA(cudaMemcpyAsync(L0.A.col.p, m->colm.p, sizeof(int32_t) * m->nnz, cudaMemcpyDeviceToDevice, s));
  DevBuf<unsigned long long> mm;
  FL_TRY(mm.reserve(2));
  const unsigned long long init[2] = {~0ull >> 1, 0ull};  // +max finite bits, 0
  FL_TRY_CUDA(cudaMemcpyAsync(mm.p, init, sizeof(init), cudaMemcpyHostToDevice, s));
  k_diag_range<<<grid_for(n, kT), kT, 0, s>>>(n, m->findrm.p, m->colm.p, H->val, mm.p);
  k_mask<<<grid_for(n, kT), kT, 0, s>>>(n, m->findrm.p, m->colm.p, H->val, H->ghost, mm.p, L0.A.val.p);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY(level_setup(L0, s));
  FL_TRY(make_sell(L0, s));
  for (int l = 0; l + 1 < kMaxLevels && H->L[l]->A.n > kMaxCoarse; ++l) {
    AmgLevel& Lv = *H->L[l];
    int nc = 0;
    FL_TRY(coarsen(Lv, l, err.p, s, &nc));
    if (nc == 0 || nc * 10 > Lv.A.n * 9) break;  // no useful coarsening left
    Csr AP;
    FL_TRY(spgemm(Lv.A, Lv.P, AP, err.p, s));
    H->L.emplace_back(new AmgLevel());
    AmgLevel& Lc = *H->L[l + 1];
    FL_TRY(spgemm(Lv.R, AP, Lc.A, err.p, s));
    FL_TRY(check_err(err.p, s, "Galerkin product row above the candidate capacity"));
    FL_TRY(level_setup(Lc, s));
  }
  // coarsest level: dense inverse
  AmgLevel& Lz = *H->L.back();
  const int nz = Lz.A.n;
  if (nz > kMaxCoarse) {
    set_error("AMG coarsening stopped at %d rows (dense coarse solve limit %d)", nz, kMaxCoarse);
    return FL_ERR_UNSUPPORTED;
  }
  std::vector<int32_t> hp(nz + 1), hc((size_t)Lz.A.nnz);
  std::vector<double> hv((size_t)Lz.A.nnz), dense((size_t)nz * nz, 0.0), inv;
  FL_TRY_CUDA(cudaMemcpyAsync(hp.data(), Lz.A.ptr.p, sizeof(int32_t) * (nz + 1), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaMemcpyAsync(hc.data(), Lz.A.col.p, sizeof(int32_t) * Lz.A.nnz, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaMemcpyAsync(hv.data(), Lz.A.val.p, sizeof(double) * Lz.A.nnz, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  for (int i = 0; i < nz; ++i)
    for (int k = hp[i]; k < hp[i + 1]; ++k) dense[(size_t)i * nz + hc[k]] += hv[k];
  // rows without any coupling (possible only when level 0 is the coarsest:
  // ghost rows) keep their diagonal, which is the ghost pivot
  FL_TRY(dense_inverse(dense, nz, inv));
  FL_TRY(H->cinv.reserve((size_t)nz * nz));
  FL_TRY_CUDA(cudaMemcpyAsync(H->cinv.p, inv.data(), sizeof(double) * nz * nz, cudaMemcpyHostToDevice, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  H->nc = nz;
  return FL_OK;
}

// K iterations of AMG-preconditioned CG (capturable; no host interaction)
void amg_iterations(fl_amg_t* H, int K, int unprec, cudaStream_t c) {
  AmgLevel& L0 = *H->L[0];
  const int n = L0.A.n, G = L0.G;
  const Op A = op_of(L0.A);
  const unsigned gv = grid_for(n, kT, 4), gl = grid_for(n, kT, 8);
  const SellOp S{n, L0.sptr.p, L0.scol.p, L0.sval.p};
  AmgState* st = H->st.p;
  (void)A;
  (void)G;
  for (int k = 0; k < K; ++k) {
    k_amg_ap_sl<<<gl, kT, 0, c>>>(S, st, H->p.p, H->w.p, H->part.p);
    k_amg_alpha<<<1, kT, 0, c>>>(st, H->part.p, (int)gl);
    k_amg_xr<<<gv, kT, 0, c>>>(n, st, H->p.p, H->w.p, H->y.p, H->r.p);
    precondition(H, H->r.p, H->z.p, c);
    const double* nv = unprec ? H->r.p : H->z.p;  // the norm of the convergence test
    k_dots<<<gv, kT, 0, c>>>(n, nv, nv, H->z.p, H->r.p, H->part.p);
    k_amg_beta<<<1, kT, 0, c>>>(st, H->part.p, (int)gv, 0, nullptr);
    k_amg_p<<<gv, kT, 0, c>>>(n, st, H->z.p, H->p.p);
  }
}

}  // namespace

extern "C" int fl_amg_create(fl_mesh m, const double* val, const uint8_t* inactive, void* stream, fl_amg* out) {
  FL_CHECK_ARG(m && val && out, "null argument");
  FL_CHECK_ARG(m->N > 0 && m->nnz > 0, "empty matrix");
  fl_amg_t* H = new fl_amg_t();
  H->m = m;
  H->val = val;
  H->ghost = inactive;
  cudaStream_t caller = stream ? (cudaStream_t)stream : m->stream;
  int st = FL_OK;
  do {
    if (cudaStreamCreateWithFlags(&H->cs, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&H->ev_in, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&H->ev_out, cudaEventDisableTiming) != cudaSuccess) {
      set_error("stream/event creation failed");
      st = FL_ERR_CUDA;
      break;
    }
    if (cudaEventRecord(H->ev_in, caller) != cudaSuccess || cudaStreamWaitEvent(H->cs, H->ev_in, 0) != cudaSuccess) {
      st = FL_ERR_CUDA;
      break;
    }
    st = build_hierarchy(H, H->cs);
  } while (0);
  if (st != FL_OK) {
    if (st == FL_ERR_CUDA && fl_last_error()[0] == 0) set_error("%s", cudaGetErrorString(cudaGetLastError()));
    cudaStreamSynchronize(H->cs);
    delete H;
    return st;
  }
  *out = H;
  return FL_OK;
}

extern "C" int fl_amg_set_norm(fl_amg H, int32_t unpreconditioned) {
  FL_CHECK_ARG(H, "null handle");
  H->unprec = unpreconditioned ? 1 : 0;
  return FL_OK;
}

extern "C" int fl_amg_set_precision(fl_amg H, int32_t fp32) {
  FL_CHECK_ARG(H, "null handle");
  if (fp32 && !H->cinvf.p) FL_TRY(make_fp32(H, H->cs));
  H->fp32 = fp32 ? 1 : 0;
  return FL_OK;
}

extern "C" int fl_amg_destroy(fl_amg H) {
  if (H) {
    cudaDeviceSynchronize();
    delete H;
  }
  return FL_OK;
}

extern "C" int fl_amg_levels(fl_amg H, int32_t* levels, int64_t* rows, int64_t* nnz, int32_t cap) {
  FL_CHECK_ARG(H && levels, "null argument");
  *levels = (int32_t)H->L.size();
  for (int l = 0; l < (int)H->L.size() && l < cap; ++l) {
    if (rows) rows[l] = H->L[l]->A.n;
    if (nnz) nnz[l] = H->L[l]->A.nnz;
  }
  return FL_OK;
}

extern "C" int fl_amg_solve(fl_amg H, const fl_solver_opts* o, const double* rhs, double* x, fl_solve_report* rep,
                            void* stream) {
  FL_CHECK_ARG(H && o && rhs && x && rep, "null argument");
  FL_CHECK_ARG(o->ksp_type == 0, "the AMG preconditioner is used with CG");
  FL_CHECK_ARG(o->precision == 0, "the AMG-preconditioned solve runs in FP64");
  FL_CHECK_ARG(o->max_its >= 0, "max_its");
  FL_CHECK_ARG(o->norm_type == 0 || o->norm_type == 1, "norm_type 0 or 1");
  // the unpreconditioned test when the handle or the options ask for it
  const int unprec = (H->unprec || o->norm_type == 1) ? 1 : 0;
  fl_mesh_t* m = H->m;
  AmgLevel& L0 = *H->L[0];
  const int n = L0.A.n, G = L0.G;
  const unsigned gs = grid_for((int64_t)n * G, kT, 8), gv = grid_for(n, kT, 4);
  const unsigned np = std::max(std::max(gs, gv), grid_for(n, kT, 8));
  FL_TRY(H->bb.reserve(n));
  FL_TRY(H->y.reserve(n));
  FL_TRY(H->r.reserve(n));
  FL_TRY(H->z.reserve(n));
  FL_TRY(H->p.reserve(n));
  FL_TRY(H->w.reserve(n));
  FL_TRY(H->part.reserve((size_t)2 * np));
  FL_TRY(H->st.reserve(1));
  FL_TRY(H->bnorm.reserve(1));
  cudaStream_t caller = stream ? (cudaStream_t)stream : m->stream;
  cudaStream_t c = H->cs;
  FL_TRY_CUDA(cudaEventRecord(H->ev_in, caller));
  FL_TRY_CUDA(cudaStreamWaitEvent(c, H->ev_in, 0));
  AmgState h{};
  h.rtol = o->rtol;
  h.atol = o->atol;
  h.dtol = o->dtol > 0 ? o->dtol : 1e5;
  h.max_its = o->max_its;
  h.guess_zero = o->start_from_zero ? 1 : 0;
  FL_TRY_CUDA(cudaMemcpyAsync(H->st.p, &h, sizeof(h), cudaMemcpyHostToDevice, c));
  AmgState* st = H->st.p;
  const Op A = op_of(L0.A);
  const Op Aorig{n, m->findrm.p, m->colm.p, H->val};
  FL_AMG_G(G, k_amg_lift, gs, c, Aorig, H->ghost, rhs, x, h.guess_zero, H->bb.p, H->y.p);
  FL_AMG_G(G, k_resid, gs, c, A, H->bb.p, H->y.p, H->r.p);
  const double* bn = nullptr;
  if (!h.guess_zero) {  // rnorm0 = ||B b|| (or ||b||) with a nonzero guess (KSPConvergedDefault)
    if (!unprec) precondition(H, H->bb.p, H->z.p, c);
    const double* v = unprec ? H->bb.p : H->z.p;
    k_dots<<<gv, kT, 0, c>>>(n, v, v, nullptr, nullptr, H->part.p);
    k_amg_norm_b<<<1, kT, 0, c>>>(H->part.p, (int)gv, H->bnorm.p);
    bn = H->bnorm.p;
  }
  precondition(H, H->r.p, H->z.p, c);
  const double* nv = unprec ? H->r.p : H->z.p;
  k_dots<<<gv, kT, 0, c>>>(n, nv, nv, H->z.p, H->r.p, H->part.p);
  k_amg_beta<<<1, kT, 0, c>>>(st, H->part.p, (int)gv, 1, bn);
  k_amg_p<<<gv, kT, 0, c>>>(n, st, H->z.p, H->p.p);
  FL_TRY_CUDA(cudaGetLastError());
  // iterations: chunks of four as one graph, replayed until done
  const int K = 4;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ex = nullptr;
  FL_TRY_CUDA(cudaStreamBeginCapture(c, cudaStreamCaptureModeThreadLocal));
  amg_iterations(H, K, unprec, c);
  cudaError_t e = cudaStreamEndCapture(c, &g);
  if (e == cudaSuccess) e = cudaGraphInstantiate(&ex, g, 0);
  if (g) cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    set_error("AMG iteration graph: %s", cudaGetErrorString(e));
    return FL_ERR_CUDA;
  }
  int st_code = FL_OK;
  for (int i = 0; i <= o->max_its; i += K) {
    if (cudaGraphLaunch(ex, c) != cudaSuccess) {
      st_code = FL_ERR_CUDA;
      break;
    }
    int done = 0;
    if (cudaMemcpyAsync(&done, &st->done, sizeof(int), cudaMemcpyDeviceToHost, c) != cudaSuccess ||
        cudaStreamSynchronize(c) != cudaSuccess) {
      st_code = FL_ERR_CUDA;
      break;
    }
    if (done) break;
  }
  cudaGraphExecDestroy(ex);
  FL_TRY(st_code);
  // true residual and the solution (ghost rows take their rhs)
  FL_AMG_G(G, k_resid, gs, c, A, H->bb.p, H->y.p, H->r.p);
  k_dots<<<gv, kT, 0, c>>>(n, H->r.p, H->r.p, H->bb.p, H->bb.p, H->part.p);
  k_amg_true<<<1, kT, 0, c>>>(st, H->part.p, (int)gv);
  k_amg_copy_back<<<gv, kT, 0, c>>>(n, H->ghost, rhs, H->y.p, x);
  FL_TRY_CUDA(cudaGetLastError());
  AmgState hs;
  FL_TRY_CUDA(cudaMemcpyAsync(&hs, st, sizeof(hs), cudaMemcpyDeviceToHost, c));
  FL_TRY_CUDA(cudaStreamSynchronize(c));
  FL_TRY_CUDA(cudaEventRecord(H->ev_out, c));
  FL_TRY_CUDA(cudaStreamWaitEvent(caller, H->ev_out, 0));
  rep->iterations = hs.its;
  rep->reason = hs.reason ? hs.reason : FL_DIVERGED_ITS;
  rep->final_rnorm = hs.rnorm;
  rep->rnorm0 = hs.rnorm0;
  rep->true_rel_residual = hs.b2 > 0 ? sqrt(hs.true_r2 / hs.b2) : sqrt(hs.true_r2);
  rep->outer_iterations = (int32_t)H->L.size();
  rep->pad = 0;
  return FL_OK;
}
