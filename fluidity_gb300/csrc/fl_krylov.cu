// fl_krylov.cu -- device Krylov solves on the assembled csr_matrix, replacing
// the PETSc KSPSolve that petsc_solve runs (femtools/Solvers.F90:1156-1302).
//
// Semantics of petsc_solve on a csr_matrix with inactive rows:
//  * inactive rows are ghost rows masked out of the PETSc numbering
//    (Petsc_Tools.F90:256-298); their columns are dropped and the rows carry
//    only the diagonal ghost_pivot = sqrt((max|d|+min|d|)*max|d|/2) over all
//    rows' |diagonal| (Petsc_Tools.F90:960-985, 1046-1056);
//  * the rhs is lifted: b = rhs - A*(rhs on ghost nodes), b = 0 on ghost rows
//    (Solvers.F90:1072-1104);
//  * the initial guess is x on active rows and 0 on ghost rows, or 0 with
//    start_from_zero (Solvers.F90:1648-1655);
//  * after the solve ghost nodes take their rhs value (Petsc_Tools.F90:726-730).
// Ghost entries of every Krylov vector stay exactly zero (b and the guess are
// zero there and the ghost rows are diagonal), so the original CSR values are
// used unchanged: ghost columns multiply zeros and ghost rows are replaced by
// pivot * x.
//
// The Krylov methods restate PETSc's KSPCG (symmetric variant) and KSPGMRES
// (left preconditioning, classical Gram-Schmidt without refinement, Givens
// rotations, happy-breakdown tolerance 1e-30), with PCJACOBI and the default
// convergence test KSPConvergedDefault on the preconditioned residual norm.
// All scalars live on the device; reductions use a fixed block partition and
// a fixed summation tree, so results are deterministic run to run.
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "fl_internal.cuh"
#include "fl_device.cuh"
#include "fl_df64.cuh"

namespace fl {

unsigned long long launches_krylov() { return unit_launches(); }

constexpr int kThreads = 256;
constexpr int kMaxRestart = 64;

// Device-resident solver state (one per solve).
struct KspState {
  // convergence test (KSPConvergedDefault)
  double rtol, atol, dtol, rnorm0, ttol, snorm_b;
  double rnorm;          // last residual norm tested
  double znorm;          // preconditioned norm ||B r|| of the last residual (CG starts)
  int its, max_its, reason, done, guess_zero;
  int unprec;            // 1: the test runs on ||r|| (KSP_NORM_UNPRECONDITIONED, CG only)
  int cg_i;              // CG iteration index (advanced on the device)
  // CG scalars
  double beta, betaold, dpi, dpiold, alpha, pcoef, dpi_next, beta_n, betaold_n;
  // ghost pivot reduction
  double mind, maxd, pivot;
  // GMRES
  int it;                // inner index of the current cycle
  int hapend;
  int live;              // the current cycle started unconverged (its correction is applied)
  int gm_first;          // next cycle is the first (device-driven restarts)
  // fp32 CG with reliable updates
  int rel, hold, outer;  // reliable mode; an update is pending; updates done
  double rmax, rdelta;   // largest recurrence residual since the last update; trigger ratio
  // true residual report
  double true_r2, b2;
  // GMRES arrays (written before they are read in every cycle, so only the
  // scalars above are uploaded and read back)
  double grs[kMaxRestart + 2];
  double cc[kMaxRestart + 1], ss[kMaxRestart + 1];
  double hh[(kMaxRestart + 1) * (kMaxRestart + 1)];   // column-major, ld = restart+1
  double lhh[kMaxRestart + 1];                        // current Gram-Schmidt coefficients
  double nrs[kMaxRestart + 1];
  double tt;
};

// An instantiated graph and the launch arguments it was captured with.
struct GraphSlot {
  cudaGraphExec_t exec = nullptr;
  std::vector<uintptr_t> key;
  ~GraphSlot() {
    if (exec) cudaGraphExecDestroy(exec);
  }
};

// Workspace cached on a mesh handle (grow-only).
struct KrylovWork {
  DevBuf<double> b, y, r, z, p, w, w2, dinv, part;
  DevBuf<double> V;     // (restart+1) * N for GMRES
  DevBuf<float> val32;  // fp32 copy of the matrix (mixed precision)
  DevBuf<float> r32, z32, p32, w32, d32, dinv32;
  DevBuf<KspState> st;
  DevBuf<unsigned> ticket;  // retire counters of the last-block reductions
  // Sliced ELL copy of the pattern for the CG SpMV: slices of 32 rows, each
  // padded to its longest row and stored column-major (entry j of the slice's
  // rows contiguous), so one thread per row reads coalesced values.
  bool sell_ready = false;
  int32_t nslices = 0;
  int64_t sell_len = 0;
  DevBuf<int32_t> swidth, sptr, scol, smap;
  DevBuf<int16_t> soff;  // column - row as int16 when every entry fits (else unused)
  bool sell16 = false;
  DevBuf<double> sval;
  DevBuf<float> sval32;
  // stream on which iteration chunks are captured and replayed as graphs
  cudaStream_t cs = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  // instantiated iteration graphs kept between solves: the FP64 CG chunk and
  // the GMRES cycle, each reused while the buffers and sizes it was captured
  // with are unchanged
  GraphSlot g_cg, g_gmres;
  // page-locked host copy of the state's scalars (the upload at the start of
  // a solve and the report read at its end are then plain DMA copies) and of
  // the cooperative GMRES's barrier flag
  struct HostPin {
    KspState st;
    unsigned long long fault;
  };
  HostPin* pin = nullptr;
  ~KrylovWork() {
    if (cs) cudaStreamDestroy(cs);
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    if (pin) cudaFreeHost(pin);
  }
};

// A chunk of solver iterations as one CUDA graph: captured on the
// workspace's own stream (the caller's stream may be the legacy default
// stream, which cannot be captured) and replayed there, ordered after the
// caller's stream by an event; end_graphs() orders the caller after it.
struct IterGraph {
  KrylovWork* W;
  cudaStream_t caller;
  cudaGraphExec_t exec = nullptr;
  bool owned = true;  // false: the exec belongs to a workspace slot
  ~IterGraph() {
    if (owned && exec) cudaGraphExecDestroy(exec);
  }
  // the graph stream starts after the work enqueued so far on the caller's
  int order_after_caller() {
    if (!W->cs) {
      FL_TRY_CUDA(cudaStreamCreateWithFlags(&W->cs, cudaStreamNonBlocking));
      FL_TRY_CUDA(cudaEventCreateWithFlags(&W->ev_in, cudaEventDisableTiming));
      FL_TRY_CUDA(cudaEventCreateWithFlags(&W->ev_out, cudaEventDisableTiming));
    }
    FL_TRY_CUDA(cudaEventRecord(W->ev_in, caller));
    FL_TRY_CUDA(cudaStreamWaitEvent(W->cs, W->ev_in, 0));
    return FL_OK;
  }
  template <class Body>
  int capture(Body body, cudaGraphExec_t* out) {
    cudaGraph_t g = nullptr;
    FL_TRY_CUDA(cudaStreamBeginCapture(W->cs, cudaStreamCaptureModeThreadLocal));
    body(W->cs);
    const cudaError_t e = cudaStreamEndCapture(W->cs, &g);
    if (e != cudaSuccess) {
      if (g) cudaGraphDestroy(g);
      set_error("iteration graph capture: %s", cudaGetErrorString(e));
      return FL_ERR_CUDA;
    }
    const cudaError_t ei = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
      *out = nullptr;
      set_error("iteration graph instantiation: %s", cudaGetErrorString(ei));
      return FL_ERR_CUDA;
    }
    return FL_OK;
  }
  template <class Body>
  int build(Body body) {
    FL_TRY(order_after_caller());
    return capture(body, &exec);
  }
  // build() through a workspace slot: the slot's graph is replayed when it
  // was captured with the same key (the launch arguments of the body)
  template <class Body>
  int build_cached(GraphSlot& slot, const std::vector<uintptr_t>& key, Body body) {
    FL_TRY(order_after_caller());
    owned = false;
    if (!slot.exec || slot.key != key) {
      if (slot.exec) cudaGraphExecDestroy(slot.exec);
      slot.exec = nullptr;
      slot.key.clear();
      FL_TRY(capture(body, &slot.exec));
      slot.key = key;
    }
    exec = slot.exec;
    return FL_OK;
  }
  int launch() {
    FL_TRY_CUDA(cudaGraphLaunch(exec, W->cs));
    return FL_OK;
  }
  // caller's stream continues after everything enqueued on the graph stream
  int join() {
    FL_TRY_CUDA(cudaEventRecord(W->ev_out, W->cs));
    FL_TRY_CUDA(cudaStreamWaitEvent(caller, W->ev_out, 0));
    return FL_OK;
  }
};

static KrylovWork* work_of(fl_mesh_t* m);

// ------------------------------------------------------------ utilities --
template <int THREADS>
__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  if (w == 0) {
    v = lane < THREADS / 32 ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  }
  __syncthreads();
  return v;  // valid in thread 0
}

// Block sum in double-float: each thread's FP64 partial is split exactly
// enough into two floats and the shuffle/shared-memory tree runs on the FP32
// pipes (a warp-wide FP64 add costs ~16 SM cycles on GB300, a double-float
// add about 3).  Result valid in thread 0, as a double.
__device__ __forceinline__ df warp_sum_df(df v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    df u;
    u.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
    u.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
    v = df_add(v, u);
  }
  return v;
}

template <int THREADS>
__device__ __forceinline__ df block_sum_dfv(df v, float2* red) {
  v = warp_sum_df(v);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = make_float2(v.hi, v.lo);
  __syncthreads();
  if (w == 0) {
    const float2 q = lane < THREADS / 32 ? red[lane] : make_float2(0.0f, 0.0f);
    v = warp_sum_df({q.x, q.y});
  }
  __syncthreads();
  return v;  // valid in thread 0
}

template <int THREADS>
__device__ __forceinline__ double block_sum_df(df v, float2* red) {
  return df_to_double(block_sum_dfv<THREADS>(v, red));
}

template <int THREADS>
__device__ __forceinline__ double block_sum_df(double v, float2* red) {
  return block_sum_df<THREADS>(df_from_double(v), red);
}

// acc + a*b in double-float: the product of the 48-bit splits of a and b
// (relative error ~2^-47), summed in double-float.  GB300 runs FP64 FMAs at
// about 1/70 of its FP32 rate (measured 1.6 per SM clock), so the Krylov dot
// products run here and the FP64 pipe keeps the vector updates and the SpMV.
__device__ __forceinline__ df df_dot_acc(df acc, double a, double b) {
  return df_add(acc, df_mul(df_from_double(a), df_from_double(b)));
}

// Exact product of two floats accumulated in double-float.
__device__ __forceinline__ df df_fma_ff(float a, float b, df acc) {
  const float p = a * b;
  const float e = fmaf(a, b, -p);
  return df_add(acc, {p, e});
}

// Sum of `n` partials in a fixed order by one block.  The partials were
// written by other blocks (possibly of the same launch), so they are read at
// L2 (__ldcg), never from this SM's L1.
__device__ double reduce_partials(const double* __restrict__ part, int n, double* red) {
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += kThreads) s += __ldcg(part + i);
  return block_sum<kThreads>(s, red);
}

// KSPConvergedDefault for iteration `it` with residual norm rn.
__device__ void converged_test(KspState& S, int it, double rn) {
  if (it == 0) {
    if (!S.guess_zero) {
      double sn = S.snorm_b;
      if (sn == 0.0) sn = rn;
      S.rnorm0 = sn;
    } else {
      S.rnorm0 = rn;
    }
    S.ttol = fmax(S.rtol * S.rnorm0, S.atol);
  }
  S.rnorm = rn;
  if (rn != rn) S.reason = FL_DIVERGED_NANORINF;
  else if (rn <= S.ttol) S.reason = rn < S.atol ? FL_CONVERGED_ATOL : FL_CONVERGED_RTOL;
  else if (rn >= S.dtol * S.rnorm0) S.reason = FL_DIVERGED_DTOL;
  if (S.reason) S.done = 1;
}

// Rows handled by a group of G lanes; the group reduces with shuffles.  All
// 32 lanes of the warp must call it together (rows past the end pass
// valid = false and contribute nothing).
template <int G>
__device__ __forceinline__ double row_dot(const int32_t* __restrict__ findrm, const int32_t* __restrict__ colm,
                                          const double* __restrict__ val, const double* __restrict__ x,
                                          int row, int sub, bool valid = true) {
  int b = 0, e = 0;
  if (valid) {
    b = __ldg(findrm + row);
    e = __ldg(findrm + row + 1);
  }
  double s = 0.0;
  for (int k = b + sub; k < e; k += G) s += __ldg(val + k) * __ldg(x + __ldg(colm + k));
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
  return s;
}


// row_dot of the gathered vector x * scale (the rounded products are the
// values of the scaled vector).
template <int G>
__device__ __forceinline__ double row_dot_scaled(const int32_t* __restrict__ findrm,
                                                 const int32_t* __restrict__ colm, const double* __restrict__ val,
                                                 const double* __restrict__ x, double scale, int row, int sub,
                                                 bool valid = true) {
  int b = 0, e = 0;
  if (valid) {
    b = __ldg(findrm + row);
    e = __ldg(findrm + row + 1);
  }
  double s = 0.0;
  for (int k = b + sub; k < e; k += G) s += __ldg(val + k) * (__ldg(x + __ldg(colm + k)) * scale);
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
  return s;
}

// ---------------------------------------------------------------- setup --
// diag / ghost pivot inputs: min and max of |diag| over all rows.
// (declared here, defined with the CG kernels)
__device__ __forceinline__ bool last_block(unsigned* ticket);

// Raw diagonal and the per-block min / max of |diagonal|; the last block to
// retire forms the ghost pivot sqrt((max + min) max / 2) from the blocks'
// partials in block order (Petsc_Tools.F90:960-985).
__global__ void k_diag(SpArgs A, const int32_t* __restrict__ centrm, double* __restrict__ dinv,
                       double* __restrict__ part_min, double* __restrict__ part_max, unsigned* ticket) {
  note_launch();
  __shared__ double rmin[kThreads / 32], rmax[kThreads / 32];
  double mn = HUGE_VAL, mx = -HUGE_VAL;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.n; i += gridDim.x * blockDim.x) {
    const int c = centrm[i];
    const double d = c >= 0 ? A.val[c] : 0.0;
    dinv[i] = d;  // raw diagonal; inverted once the pivot is known
    mn = fmin(mn, fabs(d));
    mx = fmax(mx, fabs(d));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) {
    rmin[w] = mn;
    rmax[w] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < kThreads / 32; ++k) {
      mn = fmin(mn, rmin[k]);
      mx = fmax(mx, rmax[k]);
    }
    part_min[blockIdx.x] = fmin(rmin[0], mn);
    part_max[blockIdx.x] = fmax(rmax[0], mx);
  }
  if (!last_block(ticket)) return;
  if (threadIdx.x == 0) {
    const int nb = gridDim.x;
    double pmn = HUGE_VAL, pmx = -HUGE_VAL;
    for (int k = 0; k < nb; ++k) {
      pmn = fmin(pmn, __ldcg(part_min + k));
      pmx = fmax(pmx, __ldcg(part_max + k));
    }
    KspState* st = A.st;
    st->mind = pmn;
    st->maxd = pmx;
    st->pivot = sqrt((pmx + pmn) * pmx / 2.0);
  }
}

// b = rhs - A*(rhs on ghosts) on active rows, 0 on ghost rows; y = guess;
// and the PCJACOBI inverse diagonal in place of the raw one (ghost rows: the
// pivot; a zero diagonal acts as 1, as PCSetUp_Jacobi does).
template <int G>
__global__ void k_lift(SpArgs A, const double* __restrict__ rhs, const double* __restrict__ x0, int guess_zero,
                       double* __restrict__ b, double* __restrict__ y, double* __restrict__ dinv,
                       float* __restrict__ dinv32) {
  note_launch();
  const int lane = threadIdx.x & 31, sub = lane & (G - 1);
  const int gpb = blockDim.x / G;
  for (int base = blockIdx.x * gpb; base < A.n; base += gridDim.x * gpb) {
    const int row = base + threadIdx.x / G;
    const bool valid = row < A.n;
    const bool g = valid && A.ghost && A.ghost[row];
    double s = 0.0;
    if (A.ghost) {
      int bb = 0, e = 0;
      if (valid) {
        bb = __ldg(A.findrm + row);
        e = __ldg(A.findrm + row + 1);
      }
      for (int k = bb + sub; k < e; k += G) {
        const int j = __ldg(A.colm + k);
        if (A.ghost[j]) s += A.val[k] * rhs[j];
      }
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
    }
    if (valid && sub == 0) {
      b[row] = g ? 0.0 : rhs[row] - s;
      y[row] = (guess_zero || g) ? 0.0 : x0[row];
      const double d = g ? A.st->pivot : dinv[row];
      const double v = d != 0.0 ? 1.0 / d : 1.0;
      dinv[row] = v;
      if (dinv32) dinv32[row] = (float)v;
    }
  }
}

// out = op(y) where op is the ghost-masked operator; optional fused epilogues.
// mode 0: r = b - A y, z = dinv*r, partials of z.z and of (dinv b).(dinv b)
template <int G>
__global__ void k_init_resid(SpArgs A, const double* __restrict__ b, const double* __restrict__ y,
                             const double* __restrict__ dinv, double* __restrict__ r, double* __restrict__ z,
                             double* __restrict__ part, int nparts) {
  note_launch();
  __shared__ double red[kThreads / 32];
  const int lane = threadIdx.x & 31, sub = lane & (G - 1);
  const int gpb = blockDim.x / G;
  if (A.st->done) return;  // a restart after convergence (device-driven GMRES)
  double zz = 0.0, bb = 0.0, zr = 0.0, rr = 0.0, bu = 0.0;
  const double piv = A.st->pivot;
  const bool gz = A.st->guess_zero;
  const bool unprec = A.st->unprec;
  for (int base = blockIdx.x * gpb; base < A.n; base += gridDim.x * gpb) {
    const int row = base + threadIdx.x / G;
    double ay = 0.0;
    if (!gz) ay = row_dot<G>(A.findrm, A.colm, A.val, y, row, sub, row < A.n);
    if (row < A.n && sub == 0) {
      if (A.ghost && A.ghost[row]) ay = piv * y[row];
      const double ri = b[row] - ay;
      const double zi = ri * dinv[row];
      const double bi = b[row] * dinv[row];
      r[row] = ri;
      z[row] = zi;
      zz += zi * zi;
      bb += bi * bi;
      zr += zi * ri;
      if (unprec) {
        rr += ri * ri;
        bu += b[row] * b[row];
      }
    }
  }
  zz = block_sum<kThreads>(zz, red);
  bb = block_sum<kThreads>(bb, red);
  zr = block_sum<kThreads>(zr, red);
  if (unprec) {
    rr = block_sum<kThreads>(rr, red);
    bu = block_sum<kThreads>(bu, red);
  }
  if (threadIdx.x == 0) {
    part[blockIdx.x] = zz;
    part[nparts + blockIdx.x] = bb;
    part[2 * nparts + blockIdx.x] = zr;
    if (unprec) {
      part[3 * nparts + blockIdx.x] = rr;
      part[4 * nparts + blockIdx.x] = bu;
    }
  }
}

__global__ void k_cg_start(KspState* st, const double* __restrict__ part, int nparts) {
  note_launch();
  __shared__ double red[kThreads / 32];
  const double zz = reduce_partials(part, nparts, red);
  const double bb = reduce_partials(part + nparts, nparts, red);
  const double zr = reduce_partials(part + 2 * nparts, nparts, red);
  const bool unprec = st->unprec;
  double rr = 0.0, bu = 0.0;
  if (unprec) {
    rr = reduce_partials(part + 3 * nparts, nparts, red);
    bu = reduce_partials(part + 4 * nparts, nparts, red);
  }
  if (threadIdx.x == 0) {
    KspState& S = *st;
    S.snorm_b = sqrt(unprec ? bu : bb);
    S.its = 0;
    S.reason = 0;
    S.done = 0;
    S.znorm = sqrt(zz);
    converged_test(S, 0, sqrt(unprec ? rr : zz));
    S.beta = zr;
    S.betaold = 0.0;
    S.dpi = 0.0;
    S.dpi_next = 0.0;
  }
}

// ----------------------------------------------------------- sliced ELL --
constexpr int kSlice = 32;

__global__ void k_sell_width(const int32_t* __restrict__ findrm, int n, int nslices, int32_t* __restrict__ width) {
  note_launch();
  for (int sl = blockIdx.x * blockDim.x + threadIdx.x; sl < nslices; sl += gridDim.x * blockDim.x) {
    int w = 0;
    for (int r = sl * kSlice; r < min(n, (sl + 1) * kSlice); ++r) w = max(w, findrm[r + 1] - findrm[r]);
    width[sl] = w * kSlice;  // entries of the slice
  }
}

// Column indices and CSR positions of the padded layout (padding: the row's
// own column and no CSR position).
__global__ void k_sell_fill(const int32_t* __restrict__ findrm, const int32_t* __restrict__ colm, int n,
                            const int32_t* __restrict__ sptr, int32_t* __restrict__ scol, int32_t* __restrict__ smap,
                            int16_t* __restrict__ soff, int* __restrict__ wide) {
  note_launch();
  const int nsl = (n + kSlice - 1) / kSlice;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nsl * kSlice; r += gridDim.x * blockDim.x) {
    const int sl = r / kSlice, lane = r % kSlice;
    const int w = (sptr[sl + 1] - sptr[sl]) / kSlice;
    const bool real = r < n;
    const int b = real ? findrm[r] : 0, len = real ? findrm[r + 1] - b : 0;
    for (int j = 0; j < w; ++j) {
      const int64_t idx = (int64_t)sptr[sl] + (int64_t)j * kSlice + lane;
      int c;
      if (j < len) {
        c = colm[b + j];
        smap[idx] = b + j;
      } else {
        c = real ? r : 0;
        smap[idx] = -1;
      }
      scol[idx] = c;
      const int d = real ? c - r : 0;
      if (d < -32768 || d > 32767) atomicOr(wide, 1);
      soff[idx] = (int16_t)d;
    }
  }
}

__global__ void k_sell_values(int64_t len, const int32_t* __restrict__ smap, const double* __restrict__ val,
                              double* __restrict__ sval, float* __restrict__ sval32) {
  note_launch();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < len; k += (int64_t)gridDim.x * blockDim.x) {
    const int m = smap[k];
    const double v = m >= 0 ? val[m] : 0.0;
    if (sval) sval[k] = v;
    if (sval32) sval32[k] = (float)v;
  }
}


// Row r of the sliced layout: sum over the row's entries in CSR order (the
// same order as a sequential CSR row product, so results are deterministic).
template <class V, class X>
__device__ __forceinline__ double sell_row_dot(const SellArgs& A, const V* __restrict__ sval, const X* __restrict__ x,
                                               int r) {
  const int sl = r / kSlice, lane = r % kSlice;
  const int b = __ldg(A.sptr + sl) + lane, e = __ldg(A.sptr + sl + 1);
  double s = 0.0;
  // unrolled so that several slices' value, offset and gather loads are in
  // flight together (the products are still added in slice order)
  if (A.soff) {
#pragma unroll 4
    for (int k = b; k < e; k += kSlice) s += (double)__ldg(sval + k) * (double)x[r + __ldg(A.soff + k)];
  } else {
#pragma unroll 4
    for (int k = b; k < e; k += kSlice) s += (double)__ldg(sval + k) * (double)x[__ldg(A.scol + k)];
  }
  return s;
}

// ------------------------------------------------------- CG (3 kernels) --
// One iteration i of KSPSolve_CG in three launches; each global reduction is
// finished by the last block of its launch to retire (a ticket counter), which
// sums the per-block partials in block order -- one fixed order, so results
// are deterministic -- and publishes the scalars for the next launch:
//   k_cg_p:   p = z (i == 0) or z + (beta/betaold) p
//   k_cg_ap:  w = A p; partials of p.w; last block: dpi, checks, a = beta/dpi
//   k_cg_xr:  x += a p; r -= a w; z = B r; partials of z.z and z.r;
//             last block: dp = ||z||, test, beta = z.r, checks of iteration i+1
// A launch whose state is `done` returns at once (the host polls `done`).

// True in the block that retires last; its threads then see every block's
// partials.  The counter is reset for the next launch.
__device__ __forceinline__ bool last_block(unsigned* ticket) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(ticket, 1u);
    last = (t == gridDim.x - 1);
    if (last) *ticket = 0u;
  }
  __syncthreads();
  if (last) __threadfence();
  return last;
}

__global__ void k_cg_p(int n, const KspState* st, const double* __restrict__ z, double* __restrict__ p) {
  note_launch();
  if (st->done) return;
  const int i = st->cg_i;
  const double coef = st->pcoef;
  // two rows per thread (16-byte accesses); the last odd row separately
  const int n2 = n >> 1;
  const double2* z2 = reinterpret_cast<const double2*>(z);
  double2* p2 = reinterpret_cast<double2*>(p);
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n2; k += gridDim.x * blockDim.x) {
    const double2 zv = z2[k];
    if (i == 0) {
      p2[k] = zv;
    } else {
      const double2 pv = p2[k];
      p2[k] = make_double2(zv.x + coef * pv.x, zv.y + coef * pv.y);
    }
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) p[n - 1] = i == 0 ? z[n - 1] : z[n - 1] + coef * p[n - 1];
}

__global__ void k_cg_ap(SellArgs A, const double* __restrict__ sval, const double* __restrict__ p,
                        double* __restrict__ w, double* __restrict__ part, unsigned* ticket) {
  note_launch();
  __shared__ double red[kThreads / 32];
  __shared__ float2 redf[kThreads / 32];
  KspState* st = A.st;
  if (st->done) return;
  const int i = st->cg_i;
  const double piv = st->pivot;
  df pw = {0.0f, 0.0f};
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n; row += gridDim.x * blockDim.x) {
    double s = sell_row_dot(A, sval, p, row);
    const double pi = p[row];
    if (A.ghost && A.ghost[row]) s = piv * pi;
    w[row] = s;
    pw = df_dot_acc(pw, pi, s);
  }
  const double pws = block_sum_df<kThreads>(pw, redf);
  if (threadIdx.x == 0) part[blockIdx.x] = pws;
  if (!last_block(ticket)) return;
  const double dpi = reduce_partials(part, gridDim.x, red);
  if (threadIdx.x == 0) {
    KspState& S = *st;
    S.dpiold = S.dpi;
    S.dpi = dpi;
    S.betaold = S.beta;
    if (dpi == 0.0 || (i > 0 && dpi * S.dpiold <= 0.0)) {
      S.reason = FL_DIVERGED_INDEFINITE_MAT;
      S.done = 1;
    } else {
      S.alpha = S.beta / dpi;
    }
  }
}

__global__ void k_cg_xr(int n, KspState* st, const double* __restrict__ p, const double* __restrict__ w,
                        const double* __restrict__ dinv, double* __restrict__ y, double* __restrict__ r,
                        double* __restrict__ z, double* __restrict__ part, unsigned* ticket) {
  note_launch();
  __shared__ double red[kThreads / 32];
  __shared__ float2 redf[kThreads / 32];
  if (st->done) return;
  const int i = st->cg_i;
  const double a = st->alpha;
  const bool unprec = st->unprec;
  df zz = {0.0f, 0.0f}, zr = {0.0f, 0.0f}, rr = {0.0f, 0.0f};
  // two rows per thread (16-byte accesses); the last odd row by the last thread
  const int n2 = n >> 1;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n2; k += gridDim.x * blockDim.x) {
    const double2 pv = reinterpret_cast<const double2*>(p)[k];
    const double2 wv = reinterpret_cast<const double2*>(w)[k];
    const double2 dv = reinterpret_cast<const double2*>(dinv)[k];
    const double2 rv = reinterpret_cast<const double2*>(r)[k];
    double2 yv = reinterpret_cast<double2*>(y)[k];
    yv.x += a * pv.x;
    yv.y += a * pv.y;
    const double r0 = rv.x - a * wv.x, r1 = rv.y - a * wv.y;
    const double z0 = r0 * dv.x, z1 = r1 * dv.y;
    reinterpret_cast<double2*>(y)[k] = yv;
    reinterpret_cast<double2*>(r)[k] = make_double2(r0, r1);
    reinterpret_cast<double2*>(z)[k] = make_double2(z0, z1);
    const df z0d = df_from_double(z0), z1d = df_from_double(z1);
    const df r0d = df_from_double(r0), r1d = df_from_double(r1);
    zz = df_add(zz, df_add(df_mul(z0d, z0d), df_mul(z1d, z1d)));
    zr = df_add(zr, df_add(df_mul(z0d, r0d), df_mul(z1d, r1d)));
    if (unprec) rr = df_add(rr, df_add(df_mul(r0d, r0d), df_mul(r1d, r1d)));
  }
  if ((n & 1) && blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) {
    const int k = n - 1;
    y[k] += a * p[k];
    const double rk = r[k] - a * w[k];
    const double zk = rk * dinv[k];
    r[k] = rk;
    z[k] = zk;
    zz = df_dot_acc(zz, zk, zk);
    zr = df_dot_acc(zr, zk, rk);
    rr = df_dot_acc(rr, rk, rk);
  }
  const double zzb = block_sum_df<kThreads>(zz, redf);
  const double zrb = block_sum_df<kThreads>(zr, redf);
  const double rrb = unprec ? block_sum_df<kThreads>(rr, redf) : 0.0;
  if (threadIdx.x == 0) {
    part[blockIdx.x] = zzb;
    part[gridDim.x + blockIdx.x] = zrb;
    if (unprec) part[2 * gridDim.x + blockIdx.x] = rrb;
  }
  if (!last_block(ticket)) return;
  const double zzs = reduce_partials(part, gridDim.x, red);
  const double zrs = reduce_partials(part + gridDim.x, gridDim.x, red);
  const double rrs = unprec ? reduce_partials(part + 2 * gridDim.x, gridDim.x, red) : 0.0;
  if (threadIdx.x == 0) {
    KspState& S = *st;
    // KSPConvergedDefault at iteration i+1, on ||B r|| or ||r||
    converged_test(S, i + 1, sqrt(unprec ? rrs : zzs));
    if (!S.done) {
      S.beta = zrs;
      if (i + 1 >= S.max_its) {
        S.reason = FL_DIVERGED_ITS;
        S.done = 1;
      }
    }
    if (!S.done) {
      // opening checks of iteration i+1
      S.its = i + 2;
      if (S.beta == 0.0) {
        S.reason = FL_CONVERGED_ATOL;
        S.done = 1;
        S.its = i + 2;
      } else if (S.beta * S.betaold < 0.0) {
        S.reason = FL_DIVERGED_INDEFINITE_PC;
        S.done = 1;
      }
      S.pcoef = S.beta / S.betaold;
    } else {
      S.its = i + 1;
    }
    if (!S.done) S.cg_i = i + 1;
  }
}

// Confirmation of an unpreconditioned-norm convergence on the recomputed
// residual.  k_cg_reopen lets k_init_resid form r = b - A y and z = B r from
// the iterate (done and guess_zero cleared); k_cg_confirm then keeps the
// convergence when ||b - A y|| <= ttol, or else continues CG from the same
// search direction with the recomputed residual (residual replacement: beta
// from the new z.r), so rtol bounds the true residual and not only the
// recurrence's, which drifts from it by rounding.
__global__ void k_cg_reopen(KspState* st) {
  note_launch();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  st->done = 0;
  st->guess_zero = 0;
}

__global__ void k_cg_confirm(KspState* st, const double* __restrict__ part, int nparts) {
  note_launch();
  __shared__ double red[kThreads / 32];
  const double zr = reduce_partials(part + 2 * nparts, nparts, red);
  const double rr = reduce_partials(part + 3 * nparts, nparts, red);
  if (threadIdx.x != 0) return;
  KspState& S = *st;
  const double rn = sqrt(rr);
  S.rnorm = rn;
  if (!(rn > S.ttol) || S.its >= S.max_its) {  // confirmed (or out of iterations: the reason stands)
    S.done = 1;
    return;
  }
  S.reason = 0;
  S.beta = zr;
  S.pcoef = zr / S.betaold;
  S.cg_i = S.cg_i + 1;
  S.its = S.cg_i + 1;
}

// Opening checks of iteration 0 (beta of the initial residual).
__global__ void k_cg_open(KspState* st) {
  note_launch();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  KspState& S = *st;
  S.cg_i = 0;
  if (S.done) return;
  S.its = 1;
  S.pcoef = 0.0;
  if (S.beta == 0.0) {
    S.reason = FL_CONVERGED_ATOL;
    S.done = 1;
  }
}

// --------------------------------------------------------------- GMRES --
// One Arnoldi step of KSPGMRESCycle in two launches, each global reduction
// finished by the last block to retire (last_block: block order, so the sums
// are deterministic).  The orthogonalised next vector is kept unnormalised
// in U, and the step that uses it normalises it on the fly (VecNormalize):
//   k_gmres_arnoldi: inv = 1 / ||U||; v_it = U inv on the block's rows;
//                    w = B (A v_it) (KSP_PCApplyBAorAB, left preconditioning)
//                    gathering U * inv, the same rounded values as the scaled
//                    v_it; the partials of w . v_j, j = 0..it; last block:
//                    h_j (VecMDot, classical Gram-Schmidt)
//   k_gmres_orth:    U = w - sum_j h_j v_j (VecMAXPY), partials of ||U||^2;
//                    last block: gmres_step (Hessenberg column, rotations,
//                    convergence test; ||U|| into the state)
// w is written to v_{it+1}'s slot, which the next step overwrites with the
// scaled vector; no launch reads and writes the same vector.  A launch whose
// state is `done` returns at once.
template <int G>
__global__ void __launch_bounds__(kThreads) k_gmres_arnoldi(SpArgs A, const double* __restrict__ dinv, double* V,
                                                            const double* __restrict__ U, int64_t ld, int it,
                                                            double* __restrict__ part, unsigned* ticket) {
  note_launch();
  __shared__ double sw[kThreads / G], su[kThreads / G];
  __shared__ double sacc[kMaxRestart + 1];
  KspState* st = A.st;
  if (st->done) return;
  const double piv = st->pivot;
  const double tt = st->tt;
  const double inv = tt != 0.0 ? 1.0 / tt : 1.0;
  double* vin = V + it * ld;
  double* vout = V + (it + 1) * ld;
  const int lane = threadIdx.x & 31, sub = lane & (G - 1), warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5, gpb = blockDim.x / G;
  for (int j = threadIdx.x; j <= it; j += blockDim.x) sacc[j] = 0.0;
  for (int base = blockIdx.x * gpb; base < A.n; base += gridDim.x * gpb) {
    const int row = base + threadIdx.x / G;
    double s = row_dot_scaled<G>(A.findrm, A.colm, A.val, U, inv, row, sub, row < A.n);
    if (row < A.n && sub == 0) {
      const double ui = U[row] * inv;
      if (A.ghost && A.ghost[row]) s = piv * ui;
      s *= dinv[row];
      vin[row] = ui;
      vout[row] = s;
      sw[threadIdx.x / G] = s;
      su[threadIdx.x / G] = ui;
    }
    __syncthreads();
    // the pass's rows dotted with each v_j: warp j % nw owns h_j
    const int nr = min(gpb, A.n - base);
    for (int j = warp; j <= it; j += nw) {
      const double* vj = V + j * ld + base;
      double a = 0.0;
      if (j < it) {
        for (int r = lane; r < nr; r += 32) a += sw[r] * vj[r];
      } else {
        for (int r = lane; r < nr; r += 32) a += sw[r] * su[r];
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
      if (lane == 0) sacc[j] += a;
    }
    __syncthreads();
  }
  for (int j = threadIdx.x; j <= it; j += blockDim.x) part[(int64_t)j * gridDim.x + blockIdx.x] = sacc[j];
  if (!last_block(ticket)) return;
  const int nb = gridDim.x;
  for (int j = warp; j <= it; j += nw) {
    const double* pj = part + (int64_t)j * nb;
    double a = 0.0;
    for (int b = lane; b < nb; b += 32) a += __ldcg(pj + b);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    if (lane == 0) st->lhh[j] = a;
  }
}

// Hessenberg column of iteration `it` from h_j (lhh) and ||v_{it+1}||^2 = nn,
// happy breakdown, KSPGMRESUpdateHessenberg and the convergence test (the
// body of KSPGMRESCycle after the orthogonalisation).  Called by every thread
// of one block; warp 0 works.  A dependent FP64 operation takes ~64 SM cycles
// on GB300 (a square root or a division ~650), so the serial part is kept
// short:
//  - the earlier rotations applied to the new column are the linear
//    recurrence carry_j = -s_{j-1} carry_{j-1} + c_{j-1} h_j (carry_0 = h_0,
//    rotated h_{j-1} = c_{j-1} carry_{j-1} + s_{j-1} h_j, rotated h_it =
//    carry_it), evaluated as a warp scan of the affine maps (32 rotations
//    per five shuffle steps) instead of `it` dependent steps;
//  - the happy-breakdown quotient |tt / grs| is only formed when tt < 1e-30,
//    where it can decide the test;
//  - 1 / tt (the caller's scaling, when `inv` is given) and the new rotation's
//    1 / rr come from rsqrt beside the square roots.
// The arithmetic is KSPGMRESUpdateHessenberg's up to rounding.
__device__ void gmres_step(KspState& S, double nn, int it, int restart, double* inv = nullptr) {
  __shared__ double col[kMaxRestart + 2], rc[kMaxRestart + 1], rs[kMaxRestart + 1];
  const int ld = restart + 1;
  double* hc = S.hh + (int64_t)it * ld;
  for (int j = threadIdx.x; j <= it; j += blockDim.x) col[j] = S.lhh[j];
  for (int j = threadIdx.x; j < it; j += blockDim.x) {
    rc[j] = S.cc[j];
    rs[j] = S.ss[j];
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    const double tt = sqrt(nn);
    if (lane == 0) {
      S.tt = tt;
      if (inv) *inv = nn > 0.0 ? rsqrt(nn) : 1.0;
    }
    // earlier rotations: scan of x -> A x + B over the chunk's rotations
    double carry = col[0];
    for (int c0 = 1; c0 <= it; c0 += 32) {
      const int j = c0 + lane;
      const bool act = j <= it;
      const double cj = act ? rc[j - 1] : 1.0, sj = act ? rs[j - 1] : 0.0, hj = act ? col[j] : 0.0;
      double A = act ? -sj : 1.0, B = act ? cj * hj : 0.0;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const double Ap = __shfl_up_sync(0xffffffffu, A, d), Bp = __shfl_up_sync(0xffffffffu, B, d);
        if (lane >= d) {
          B = fma(A, Bp, B);
          A = A * Ap;
        }
      }
      const double cur = fma(A, carry, B);  // carry_j
      double prev = __shfl_up_sync(0xffffffffu, cur, 1);
      if (lane == 0) prev = carry;
      __syncwarp();
      if (act) col[j - 1] = fma(cj, prev, sj * hj);
      carry = __shfl_sync(0xffffffffu, cur, min(31, it - c0));
      __syncwarp();
    }
    if (lane == 0) {
      col[it] = carry;
      col[it + 1] = tt;
      // hapbnd = min(|tt / grs(it)|, 1e-30); hapend = tt < hapbnd
      const bool hapend = tt < 1e-30 && tt < fabs(tt / S.grs[it]);
      bool null_col = false;
      double res = 0.0;
      if (!hapend) {
        const double h0 = carry, h1 = tt;
        const double r2 = h0 * h0 + h1 * h1;
        if (r2 == 0.0) {
          S.reason = FL_DIVERGED_NULL;
          S.done = 1;
          S.it = it;  // this column is not used
          null_col = true;
        } else {
          const double ri = rsqrt(r2);
          const double c = h0 * ri, sn = h1 * ri;
          S.cc[it] = c;
          S.ss[it] = sn;
          const double g = S.grs[it];
          S.grs[it + 1] = -(sn * g);
          S.grs[it] = c * g;
          col[it] = c * h0 + sn * h1;
          res = fabs(S.grs[it + 1]);
        }
      }
      if (!null_col) {
        S.it = it + 1;
        S.its += 1;
        converged_test(S, S.its, res);
        if (hapend && !S.reason) {
          S.reason = FL_DIVERGED_BREAKDOWN;
          S.done = 1;
        }
        if (!S.done && S.its >= S.max_its) {
          S.reason = FL_DIVERGED_ITS;  // KSPSolve_GMRES: itcount >= max_it
          S.done = 1;
        }
      }
    }
  }
  __syncthreads();
  for (int j = threadIdx.x; j <= it + 1; j += blockDim.x) hc[j] = col[j];
}

__global__ void __launch_bounds__(kThreads) k_gmres_orth(int n, KspState* st, const double* __restrict__ V,
                                                         double* __restrict__ U, int64_t ld, int it, int restart,
                                                         double* __restrict__ part, unsigned* ticket) {
  note_launch();
  __shared__ double red[kThreads / 32];
  __shared__ double sh[kMaxRestart + 1];
  if (st->done) return;
  for (int j = threadIdx.x; j <= it; j += blockDim.x) sh[j] = st->lhh[j];
  __syncthreads();
  const double* vn = V + (int64_t)(it + 1) * ld;
  double nn = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    // subtraction order j = 0..it; the loads of four basis vectors are
    // issued together
    double s = vn[i];
    int j = 0;
    for (; j + 3 <= it; j += 4) {
      const double a0 = V[(int64_t)j * ld + i], a1 = V[(int64_t)(j + 1) * ld + i];
      const double a2 = V[(int64_t)(j + 2) * ld + i], a3 = V[(int64_t)(j + 3) * ld + i];
      s -= sh[j] * a0;
      s -= sh[j + 1] * a1;
      s -= sh[j + 2] * a2;
      s -= sh[j + 3] * a3;
    }
    for (; j <= it; ++j) s -= sh[j] * V[(int64_t)j * ld + i];
    U[i] = s;
    nn += s * s;
  }
  nn = block_sum<kThreads>(nn, red);
  if (threadIdx.x == 0) part[blockIdx.x] = nn;
  if (!last_block(ticket)) return;
  nn = reduce_partials(part, gridDim.x, red);
  gmres_step(*st, nn, it, restart);
}

// Cycle start: res = ||v0||, grs(0) = res, test; v0 normalised.  first < 0
// takes the first-cycle flag from the state (restarts decided on the device);
// a solve that has already converged leaves the state as it is.
__global__ void k_gmres_cycle_start(KspState* st, const double* __restrict__ part, int nparts, int first) {
  note_launch();
  __shared__ double red[kThreads / 32];
  if (st->done) {
    __syncthreads();
    if (threadIdx.x == 0) st->live = 0;
    return;
  }
  const double nn = reduce_partials(part, nparts, red);
  const double bb = reduce_partials(part + nparts, nparts, red);
  if (threadIdx.x != 0) return;
  KspState& S = *st;
  if (first < 0) {
    first = S.gm_first;
    S.gm_first = 0;
  }
  S.live = 1;
  const double res = sqrt(nn);
  if (first) {
    S.snorm_b = sqrt(bb);
    S.its = 0;
    S.reason = 0;
    S.done = 0;
  }
  S.grs[0] = res;
  S.it = 0;
  S.hapend = 0;
  S.tt = res;
  if (res == 0.0) {
    S.reason = FL_CONVERGED_ATOL;
    S.done = 1;
    S.rnorm = 0.0;
    if (first) S.rnorm0 = 0.0;
    return;
  }
  converged_test(S, S.its, res);
}

// Partials of ||v0||^2 and ||B b||^2 for the cycle start.
__global__ void k_norm2_pair(int n, const double* __restrict__ v, const double* __restrict__ b,
                             const double* __restrict__ dinv, double* __restrict__ part, int nparts) {
  note_launch();
  __shared__ double red[kThreads / 32];
  double a = 0.0, c = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    a += v[i] * v[i];
    const double bi = b[i] * dinv[i];
    c += bi * bi;
  }
  a = block_sum<kThreads>(a, red);
  c = block_sum<kThreads>(c, red);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = a;
    part[nparts + blockIdx.x] = c;
  }
}

// KSPGMRESBuildSoln: back substitution on the rotated Hessenberg system, one
// warp: lane l keeps the right-hand sides t_l, t_{l+32}; after nrs_k is
// known every row above it subtracts H(i,k) nrs_k (column k of H is
// contiguous, so each step is one coalesced load).
__device__ void gmres_backsolve_warp(KspState& S, int restart) {
  const int ld = restart + 1;
  const int last = S.it - 1;
  if (last < 0) return;
  const int lane = threadIdx.x & 31;
  double t0 = lane <= last ? S.grs[lane] : 0.0;
  double t1 = lane + 32 <= last ? S.grs[lane + 32] : 0.0;
  for (int k = last; k >= 0; --k) {
    const double* hk = S.hh + (int64_t)k * ld;
    const double h0 = lane < k ? hk[lane] : 0.0;
    const double h1 = lane + 32 < k ? hk[lane + 32] : 0.0;
    const double tk = __shfl_sync(0xffffffffu, k < 32 ? t0 : t1, k & 31);
    const double hkk = hk[k];
    const double y = hkk != 0.0 ? tk / hkk : 0.0;
    if (lane == 0) S.nrs[k] = y;
    t0 -= h0 * y;
    t1 -= h1 * y;
  }
}

__global__ void k_gmres_backsolve(KspState* st, int restart) {
  note_launch();
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  if (!st->live) return;
  gmres_backsolve_warp(*st, restart);
}

__global__ void k_gmres_update_x(int n, const KspState* st, const double* __restrict__ V, int64_t ld,
                                 double* __restrict__ y) {
  note_launch();
  __shared__ double sy[kMaxRestart + 1];
  if (!st->live) return;
  const int last = st->it - 1;
  if (last < 0) return;
  for (int j = threadIdx.x; j <= last; j += blockDim.x) sy[j] = st->nrs[j];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s = 0.0;
    int j = 0;
    for (; j + 3 <= last; j += 4) {
      const double a0 = V[(int64_t)j * ld + i], a1 = V[(int64_t)(j + 1) * ld + i];
      const double a2 = V[(int64_t)(j + 2) * ld + i], a3 = V[(int64_t)(j + 3) * ld + i];
      s += sy[j] * a0;
      s += sy[j + 1] * a1;
      s += sy[j + 2] * a2;
      s += sy[j + 3] * a3;
    }
    for (; j <= last; ++j) s += sy[j] * V[(int64_t)j * ld + i];
    y[i] += s;
  }
}

// End of a device-driven cycle: the iteration limit (KSPSolve_GMRES's
// itcount >= max_it test) and the nonzero guess of the restart.
__global__ void k_gmres_cycle_end(KspState* st) {
  note_launch();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  KspState& S = *st;
  if (!S.live) return;
  S.live = 0;
  if (!S.done && S.its >= S.max_its) {
    S.reason = FL_DIVERGED_ITS;
    S.done = 1;
  }
  S.guess_zero = 0;
}

// ------------------------------------------- GMRES in one cooperative launch --
// The whole of KSPSolve_GMRES for a small system in one launch, for systems
// where a launch per Arnoldi phase costs more than the phase.  Each block
// owns fixed rows (passes of kThreads / PG rows, PG lanes per row: row group
// blockIdx.x + k nb) and keeps their slice of the Krylov basis in shared
// memory, so only the SpMV gathers and the reduction partials cross blocks.
// Every block also keeps an identical copy of the solver state in shared
// memory: after each grid barrier every block sums the same partials in the
// same order, so all copies take the same decisions (convergence, restarts)
// without a broadcast.  One Arnoldi step is two phases and two barriers:
//   A: w = B A v_it on the block's rows, gathering the unnormalised U and
//      scaling the row sums by inv = 1 / ||U||; the rows of v_it = U inv
//      stored; the block's partials of w . v_j, j <= it
//   B: h_j from the partials; U = w - sum_j h_j v_j (VecMAXPY) on the
//      block's rows, published for the next gathers; partials of ||U||^2
//   then every block: tt = ||U||, the Hessenberg column, rotations and the
//   convergence test (gmres_step).
// FP64 latency shapes the layout (a dependent FP64 operation ~64 SM cycles
// on GB300): short FMA chains (PG lanes per row; dot products lane-per-basis-
// vector over a warp's rows, then a tree over the warps), and the cross-block
// partials published and summed in double-float on the FP32 pipes.  The
// Krylov space and the tests are KSPGMRESCycle's; the sums run in another
// order than the launch-per-phase schedule's, so results agree to rounding.
// Data that other blocks write during the launch (U, y, the partials) is
// read at L2 (__ldcg).
constexpr unsigned long long kBarrierWaitNs = 1000000000ull;  // a grid barrier gives up after 1 s
// PG lanes per row: the host takes the most (8, 4, 2) that keep the row
// groups of kThreads / PG rows within one per SM, so that a block makes one
// pass where it can (measured: 4,913 rows best at 4, 15,625 and 35,937 at 2).

struct PersistArgs {
  SpArgs A;                      // A.st: the global state (read at the start, published at the end)
  const double* dinv;            // Jacobi inverse diagonal (ghost rows 1 / pivot)
  const double* b;               // right-hand side with the ghost rows lifted
  double* y;                     // iterate
  double* U;                     // unnormalised next basis vector (gathered by the SpMV)
  float2* part;                  // double-float partials: (kMaxRestart + 1) * nb of h, then 2 * nb
  unsigned long long* bar;       // [0] arrivals (monotonic), [1] error flag
  int restart;
  int npass;                     // row passes per block
  int withhold;                  // failure-injection test: this block never arrives (-1: none)
  unsigned long long wait_ns;    // limit of one barrier wait
};

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long atom_add_acq_rel_u64(unsigned long long* p, unsigned long long v) {
  unsigned long long old;
  asm volatile("atom.acq_rel.gpu.global.add.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
  return old;
}

// Barrier over the blocks of a cooperative launch (all co-resident): an
// arrival counter that only grows, barrier k complete once it reaches k nb.
// The block's writes are ordered before its arrival by __syncthreads and the
// release half of the atomic; the acquiring load orders the reads after.  The
// wait is bounded: after wait_ns (kBarrierWaitNs unless a test shortens it),
// or once another block has raised the error flag, the block raises the flag
// and every thread gets false (the caller leaves its loops and returns; the
// host reads the flag).
__device__ bool grid_barrier(unsigned long long* bar, unsigned long long wait_ns) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int good = 1;
    const unsigned long long nb = gridDim.x;
    const unsigned long long old = atom_add_acq_rel_u64(bar, 1ull);
    const unsigned long long target = (old / nb + 1) * nb;
    if (old + 1 < target) {
      const unsigned long long t0 = global_ns();
      while (ld_acquire_u64(bar) < target) {
        if (global_ns() - t0 > wait_ns || ld_acquire_u64(bar + 1) != 0ull) {
          atomicExch(bar + 1, 1ull);
          good = 0;
          break;
        }
      }
    }
    ok = good;
  }
  __syncthreads();
  return ok != 0;
}

// Row sum of A x over G lanes, x read at L2.
template <int G>
__device__ __forceinline__ double row_dot_cg(const int32_t* __restrict__ findrm, const int32_t* __restrict__ colm,
                                             const double* __restrict__ val, const double* x, int row, int sub,
                                             bool valid) {
  int b = 0, e = 0;
  if (valid) {
    b = __ldg(findrm + row);
    e = __ldg(findrm + row + 1);
  }
  double s = 0.0;
  for (int k = b + sub; k < e; k += G) s = fma(__ldg(val + k), __ldcg(x + __ldg(colm + k)), s);
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, G);
  return s;
}

__device__ __forceinline__ float2 df_pack(df v) { return make_float2(v.hi, v.lo); }

// Shared memory of k_gmres_persistent beyond its static arrays: the block's
// rows of v_0..v_restart (row stride rows + 1, odd, so lanes reading one row
// of different vectors fall in different banks), of w and of U (rows past N
// hold zeros).
inline size_t persist_smem_bytes(int restart, int npass, int pg) {
  const size_t rows = (size_t)npass * (kThreads / pg);
  return ((size_t)(restart + 1) * (rows + 1) + 2 * rows) * sizeof(double);
}

template <int PG>
__global__ void __launch_bounds__(kThreads, 1) k_gmres_persistent(PersistArgs P) {
  constexpr int kPG = PG, kPRows = kThreads / PG;
  note_launch();
  __shared__ KspState S;
  __shared__ float2 redf[kThreads / 32];
  __shared__ double red8[kThreads / 32][2 * 32];  // dot partials of the warps, j < 64
  __shared__ double sred[2];
  __shared__ double sinv;
  extern __shared__ double dyn[];
  const SpArgs& A = P.A;
  const int n = A.n, nb = gridDim.x, restart = P.restart;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, nw = blockDim.x >> 5;
  const int sub = lane & (kPG - 1);
  const int rows = P.npass * kPRows, vs = rows + 1;
  double* Vs = dyn;  // [j * vs + lr]; local row lr = k kPRows + r <-> row (blockIdx.x + k nb) kPRows + r
  double* Ws = dyn + (size_t)(restart + 1) * vs;
  double* Us = Ws + rows;
  double* U = P.U;
  float2* part_h = P.part;                                    // [j * nb + b]
  float2* part_n = P.part + (int64_t)(kMaxRestart + 1) * nb;  // [b], [nb + b]
  auto grow = [&](int lr) { return (blockIdx.x + (lr / kPRows) * nb) * kPRows + lr % kPRows; };
  if ((int)blockIdx.x == P.withhold) return;  // failure-injection test: the others' first barrier runs out
  {
    const int* src = reinterpret_cast<const int*>(A.st);
    int* dst = reinterpret_cast<int*>(&S);
    for (int k = tid; k < (int)(offsetof(KspState, grs) / sizeof(int)); k += blockDim.x) dst[k] = src[k];
  }
  __syncthreads();
  const double piv = S.pivot;
  bool ok = true;
  for (int cycle = 0; ok && cycle <= S.max_its; ++cycle) {
    // KSPInitialResidual: U = B (b - A y) (zero guess: B b); ||U||^2, ||B b||^2
    const bool gz = S.guess_zero;
    double zz = 0.0, bb = 0.0;
    for (int k = 0; k < P.npass; ++k) {
      const int lr = k * kPRows + tid / kPG, row = grow(lr);
      double ay = 0.0;
      if (!gz) ay = row_dot_cg<kPG>(A.findrm, A.colm, A.val, P.y, row, sub, row < n);
      if (sub == 0) {
        double zi = 0.0;
        if (row < n) {
          if (A.ghost && A.ghost[row]) ay = piv * __ldcg(P.y + row);
          const double bi0 = P.b[row], di = P.dinv[row];
          zi = (bi0 - ay) * di;
          const double bi = bi0 * di;
          U[row] = zi;
          zz = fma(zi, zi, zz);
          bb = fma(bi, bi, bb);
        }
        Us[lr] = zi;
      }
    }
    {
      const df zs = block_sum_dfv<kThreads>(df_from_double(zz), redf);
      const df bs = block_sum_dfv<kThreads>(df_from_double(bb), redf);
      if (tid == 0) {
        part_n[blockIdx.x] = df_pack(zs);
        part_n[nb + blockIdx.x] = df_pack(bs);
      }
    }
    if (!(ok = grid_barrier(P.bar, P.wait_ns))) break;
    {
      // the cycle start of k_gmres_cycle_start, on every block's copy
      if (warp < 2) {
        const float2* p = part_n + warp * nb;
        df a = {0.0f, 0.0f};
        for (int b = lane; b < nb; b += 32) {
          const float2 q = __ldcg(p + b);
          a = df_add(a, {q.x, q.y});
        }
        a = warp_sum_df(a);
        if (lane == 0) sred[warp] = df_to_double(a);
      }
      __syncthreads();
      if (tid == 0) {
        const int first = S.gm_first;
        S.gm_first = 0;
        const double res = sqrt(sred[0]);
        if (first) {
          S.snorm_b = sqrt(sred[1]);
          S.its = 0;
          S.reason = 0;
          S.done = 0;
        }
        S.grs[0] = res;
        S.it = 0;
        S.hapend = 0;
        S.tt = res;
        if (res == 0.0) {
          S.reason = FL_CONVERGED_ATOL;
          S.done = 1;
          S.rnorm = 0.0;
          if (first) S.rnorm0 = 0.0;
        } else {
          converged_test(S, S.its, res);
        }
        sinv = res != 0.0 ? 1.0 / res : 1.0;
      }
      __syncthreads();
    }
    for (int it = 0; it < restart && !S.done; ++it) {
      // phase A: w = B A v_it on the block's rows, v_it's rows scaled
      const double inv = sinv;
      double* Vi = Vs + (size_t)it * vs;
      for (int k = 0; k < P.npass; ++k) {
        const int lr = k * kPRows + tid / kPG, row = grow(lr);
        double s = row_dot_cg<kPG>(A.findrm, A.colm, A.val, U, row, sub, row < n);
        if (sub == 0) {
          const double ui = Us[lr] * inv;
          if (row < n) {
            s = (A.ghost && A.ghost[row]) ? piv * ui : s * inv;
            s *= P.dinv[row];
          } else {
            s = 0.0;
          }
          Ws[lr] = s;
          Vi[lr] = ui;
        }
      }
      __syncthreads();
      // partials of w . v_j: lane j (and j + 32) over the warp's rows, then
      // a tree over the warps
      {
        const int cr = rows / nw;
        double a0 = 0.0, a1 = 0.0;
        for (int lr = warp * cr; lr < (warp + 1) * cr; ++lr) {
          const double wr = Ws[lr];
          if (lane <= it) a0 = fma(wr, Vs[(size_t)lane * vs + lr], a0);
          if (lane + 32 <= it) a1 = fma(wr, Vs[(size_t)(lane + 32) * vs + lr], a1);
        }
        red8[warp][lane] = a0;
        red8[warp][lane + 32] = a1;
        __syncthreads();
        const int j = tid & 63, w2 = tid >> 6;
        red8[w2][j] += red8[w2 + 4][j];
        __syncthreads();
        if (tid < 128) red8[w2][j] += red8[w2 + 2][j];
        __syncthreads();
        if (tid < 64 && j <= it) part_h[(int64_t)j * nb + blockIdx.x] = df_pack(df_from_double(red8[0][j] + red8[1][j]));
      }
      if (!(ok = grid_barrier(P.bar, P.wait_ns))) break;
      // phase B: h_j (classical Gram-Schmidt): warp j % nw sums the blocks'
      // partials of h_j, four j at a time
      for (int j0 = warp; j0 <= it; j0 += 4 * nw) {
        df a[4] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
        for (int b = lane; b < nb; b += 32) {
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int j = j0 + q * nw;
            if (j <= it) {
              const float2 v = __ldcg(part_h + (int64_t)j * nb + b);
              a[q] = df_add(a[q], {v.x, v.y});
            }
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const df t = warp_sum_df(a[q]);
          if (lane == 0 && j0 + q * nw <= it) S.lhh[j0 + q * nw] = df_to_double(t);
        }
      }
      __syncthreads();
      // U = w - sum_j h_j v_j: kPG threads per row, thread sub takes j = sub (mod kPG)
      double nn = 0.0;
      for (int k = 0; k < P.npass; ++k) {
        const int lr = k * kPRows + tid / kPG, row = grow(lr);
        double sum = 0.0;
        for (int j = sub; j <= it; j += kPG) sum = fma(S.lhh[j], Vs[(size_t)j * vs + lr], sum);
#pragma unroll
        for (int o = kPG / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, kPG);
        if (sub == 0) {
          double u = 0.0;
          if (row < n) {
            u = Ws[lr] - sum;
            U[row] = u;
          }
          Us[lr] = u;
          nn = fma(u, u, nn);
        }
      }
      {
        const df ns = block_sum_dfv<kThreads>(df_from_double(nn), redf);
        if (tid == 0) part_n[blockIdx.x] = df_pack(ns);
      }
      if (!(ok = grid_barrier(P.bar, P.wait_ns))) break;
      // every block: ||U||, Hessenberg column, rotations, convergence test
      if (warp == 0) {
        df a = {0.0f, 0.0f};
        for (int b = lane; b < nb; b += 32) {
          const float2 q = __ldcg(part_n + b);
          a = df_add(a, {q.x, q.y});
        }
        a = warp_sum_df(a);
        if (lane == 0) sred[0] = df_to_double(a);
      }
      __syncthreads();
      gmres_step(S, sred[0], it, restart, &sinv);
    }
    if (!ok) break;
    // KSPGMRESBuildSoln: y += V nrs on the block's rows
    if (S.it > 0) {
      if (warp == 0) gmres_backsolve_warp(S, restart);
      __syncthreads();
      const int last = S.it - 1;
      for (int k = 0; k < P.npass; ++k) {
        const int lr = k * kPRows + tid / kPG, row = grow(lr);
        double sum = 0.0;
        for (int j = sub; j <= last; j += kPG) sum = fma(S.nrs[j], Vs[(size_t)j * vs + lr], sum);
#pragma unroll
        for (int o = kPG / 2; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o, kPG);
        if (sub == 0 && row < n) P.y[row] = __ldcg(P.y + row) + sum;
      }
    }
    // cycle end: KSPSolve_GMRES's itcount >= max_it; the restart's guess is nonzero
    if (tid == 0) {
      if (!S.done && S.its >= S.max_its) {
        S.reason = FL_DIVERGED_ITS;
        S.done = 1;
      }
      S.guess_zero = 0;
    }
    __syncthreads();
    if (S.done) break;
    if (!(ok = grid_barrier(P.bar, P.wait_ns))) break;
  }
  // publish the scalars (every copy is the same; block 0 writes them)
  if (blockIdx.x == 0) {
    if (tid == 0 && !ok) S.done = 1;
    __syncthreads();
    const int* src = reinterpret_cast<const int*>(&S);
    int* dst = reinterpret_cast<int*>(A.st);
    for (int k = tid; k < (int)(offsetof(KspState, grs) / sizeof(int)); k += blockDim.x) dst[k] = src[k];
  }
}

// ------------------------------------------------------------- finalise --
template <int G>
// ||b - A y||^2 and ||b||^2 (the report's true residual), the last block
// summing the partials in block order; and x = y on active rows, the rhs on
// ghost rows (Petsc_Tools.F90:726-730).
__global__ void k_true_resid(SpArgs A, const double* __restrict__ b, const double* __restrict__ y,
                             double* __restrict__ part, int nparts, const double* __restrict__ rhs,
                             double* __restrict__ x, unsigned* ticket) {
  note_launch();
  __shared__ double red[kThreads / 32];
  const double piv = A.st->pivot;
  const int lane = threadIdx.x & 31, sub = lane & (G - 1);
  const int gpb = blockDim.x / G;
  double rr = 0.0, bb = 0.0;
  for (int base = blockIdx.x * gpb; base < A.n; base += gridDim.x * gpb) {
    const int row = base + threadIdx.x / G;
    double s = 0.0;
    s = row_dot<G>(A.findrm, A.colm, A.val, y, row, sub, row < A.n);
    if (row < A.n && sub == 0) {
      const bool g = A.ghost && A.ghost[row];
      if (g) s = piv * y[row];
      const double ri = b[row] - s;
      rr += ri * ri;
      bb += b[row] * b[row];
      x[row] = g ? rhs[row] : y[row];
    }
  }
  rr = block_sum<kThreads>(rr, red);
  bb = block_sum<kThreads>(bb, red);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = rr;
    part[nparts + blockIdx.x] = bb;
  }
  if (!last_block(ticket)) return;
  rr = reduce_partials(part, nparts, red);
  bb = reduce_partials(part + nparts, nparts, red);
  if (threadIdx.x == 0) {
    A.st->true_r2 = rr;
    A.st->b2 = bb;
  }
}

// ----------------------------------------------------------- mixed (fp32) --
// Inner CG in fp32 storage (matrix, vectors) with fp64 dot products, driven
// by an fp64 iterative-refinement loop on the true residual.
__global__ void k_to_f32(int64_t n, const double* __restrict__ a, float* __restrict__ b) {
  note_launch();
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

struct SpArgs32 {
  int32_t n;
  const int32_t* findrm;
  const int32_t* colm;
  const float* val;
  const uint8_t* ghost;
};

// Inner CG of the refinement, same three-launch structure as the FP64 CG:
// fp32 matrix and vectors, fp64 dot products and scalars.  The inner problem
// starts from d = 0 and stops when ||B r|| <= ttol (set by the outer loop).
__global__ void k_cg32_p(int n, const KspState* st, const float* __restrict__ z, float* __restrict__ p) {
  note_launch();
  if (st->done || st->hold) return;
  const int i = st->cg_i;
  const float coef = (float)st->pcoef;
  // four rows per thread (16-byte accesses); the last n % 4 rows by thread 0
  const int n4 = n >> 2;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += gridDim.x * blockDim.x) {
    const float4 zv = reinterpret_cast<const float4*>(z)[k];
    if (i == 0) {
      reinterpret_cast<float4*>(p)[k] = zv;
    } else {
      const float4 pv = reinterpret_cast<const float4*>(p)[k];
      reinterpret_cast<float4*>(p)[k] = make_float4(fmaf(coef, pv.x, zv.x), fmaf(coef, pv.y, zv.y),
                                                    fmaf(coef, pv.z, zv.z), fmaf(coef, pv.w, zv.w));
    }
  }
  if (blockIdx.x == 0 && threadIdx.x == 0)
    for (int k = n4 * 4; k < n; ++k) p[k] = i == 0 ? z[k] : fmaf(coef, p[k], z[k]);
}

__global__ void k_cg32_ap(SellArgs A, const float* __restrict__ sval, float piv, const float* __restrict__ p,
                          float* __restrict__ w, double* __restrict__ part, unsigned* ticket) {
  note_launch();
  __shared__ double red[kThreads / 32];
  __shared__ float2 redf[kThreads / 32];
  KspState* st = A.st;
  if (st->done || st->hold) return;
  df pwd = {0.0f, 0.0f};
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < A.n; row += gridDim.x * blockDim.x) {
    const int sl = row / kSlice, lane = row % kSlice;
    const int b = __ldg(A.sptr + sl) + lane, e = __ldg(A.sptr + sl + 1);
    float s = 0.0f;
    if (A.soff) {
      // eight slices at a time: their offsets and values first, then the
      // eight gathers, then the products added in slice order
      int k = b;
      for (; k + 7 * kSlice < e; k += 8 * kSlice) {
        float a[8];
        int c[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          a[u] = __ldg(sval + k + u * kSlice);
          c[u] = row + __ldg(A.soff + k + u * kSlice);
        }
        float xv[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) xv[u] = p[c[u]];
#pragma unroll
        for (int u = 0; u < 8; ++u) s = fmaf(a[u], xv[u], s);
      }
      for (; k < e; k += kSlice) s = fmaf(__ldg(sval + k), p[row + __ldg(A.soff + k)], s);
    } else {
#pragma unroll 4
      for (int k = b; k < e; k += kSlice) s = fmaf(__ldg(sval + k), p[__ldg(A.scol + k)], s);
    }
    const float pi = p[row];
    if (A.ghost && A.ghost[row]) s = piv * pi;
    w[row] = s;
    pwd = df_fma_ff(pi, s, pwd);
  }
  const double pw = block_sum_df<kThreads>(pwd, redf);
  if (threadIdx.x == 0) part[blockIdx.x] = pw;
  if (!last_block(ticket)) return;
  const double dpi = reduce_partials(part, gridDim.x, red);
  if (threadIdx.x == 0) {
    KspState& S = *st;
    S.betaold = S.beta;
    if (dpi <= 0.0 || dpi != dpi) {
      S.reason = FL_DIVERGED_INDEFINITE_MAT;  // inner breakdown: the outer loop decides
      S.done = 1;
    } else {
      S.alpha = S.beta / dpi;
    }
  }
}

__global__ void k_cg32_xr(int n, KspState* st, const float* __restrict__ p, const float* __restrict__ w,
                          const float* __restrict__ dinv, float* __restrict__ d, float* __restrict__ r,
                          float* __restrict__ z, double* __restrict__ part, unsigned* ticket) {
  note_launch();
  __shared__ double red[kThreads / 32];
  if (st->done || st->hold) return;
  __shared__ float2 redf[kThreads / 32];
  const int i = st->cg_i;
  const float a = (float)st->alpha;
  // reliable updates with the unpreconditioned test trigger on ||r|| as well
  const bool unprec = st->rel && st->unprec;
  df zzd = {0.0f, 0.0f}, zrd = {0.0f, 0.0f}, rrd = {0.0f, 0.0f};
  // four rows per thread (16-byte accesses); the last n % 4 rows by the last thread
  const int n4 = n >> 2;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += gridDim.x * blockDim.x) {
    const float4 pv = reinterpret_cast<const float4*>(p)[k];
    const float4 wv = reinterpret_cast<const float4*>(w)[k];
    const float4 dv = reinterpret_cast<const float4*>(dinv)[k];
    const float4 rv = reinterpret_cast<const float4*>(r)[k];
    const float4 cv = reinterpret_cast<const float4*>(d)[k];
    const float pa[4] = {pv.x, pv.y, pv.z, pv.w}, wa[4] = {wv.x, wv.y, wv.z, wv.w};
    const float da[4] = {dv.x, dv.y, dv.z, dv.w}, ra[4] = {rv.x, rv.y, rv.z, rv.w};
    const float ca[4] = {cv.x, cv.y, cv.z, cv.w};
    float ro[4], zo[4], co[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      co[u] = fmaf(a, pa[u], ca[u]);
      ro[u] = fmaf(-a, wa[u], ra[u]);
      zo[u] = ro[u] * da[u];
      zzd = df_fma_ff(zo[u], zo[u], zzd);
      zrd = df_fma_ff(zo[u], ro[u], zrd);
      if (unprec) rrd = df_fma_ff(ro[u], ro[u], rrd);
    }
    reinterpret_cast<float4*>(d)[k] = make_float4(co[0], co[1], co[2], co[3]);
    reinterpret_cast<float4*>(r)[k] = make_float4(ro[0], ro[1], ro[2], ro[3]);
    reinterpret_cast<float4*>(z)[k] = make_float4(zo[0], zo[1], zo[2], zo[3]);
  }
  if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1)
    for (int k = n4 * 4; k < n; ++k) {
      d[k] = fmaf(a, p[k], d[k]);
      const float rk = fmaf(-a, w[k], r[k]);
      const float zk = rk * dinv[k];
      r[k] = rk;
      z[k] = zk;
      zzd = df_fma_ff(zk, zk, zzd);
      zrd = df_fma_ff(zk, rk, zrd);
      rrd = df_fma_ff(rk, rk, rrd);
    }
  const double zz = block_sum_df<kThreads>(zzd, redf);
  const double zr = block_sum_df<kThreads>(zrd, redf);
  const double rr = unprec ? block_sum_df<kThreads>(rrd, redf) : 0.0;
  if (threadIdx.x == 0) {
    part[blockIdx.x] = zz;
    part[gridDim.x + blockIdx.x] = zr;
    if (unprec) part[2 * gridDim.x + blockIdx.x] = rr;
  }
  if (!last_block(ticket)) return;
  const double zzs = reduce_partials(part, gridDim.x, red);
  const double zrs = reduce_partials(part + gridDim.x, gridDim.x, red);
  const double rrs = unprec ? reduce_partials(part + 2 * gridDim.x, gridDim.x, red) : 0.0;
  if (threadIdx.x == 0) {
    KspState& S = *st;
    S.its = i + 1;
    S.rnorm = sqrt(unprec ? rrs : zzs);
    if (!(S.rnorm == S.rnorm)) {
      S.reason = FL_DIVERGED_NANORINF;
      S.done = 1;
    } else if (S.rel) {
      // reliable updates: the recurrence residual is only a trigger; the
      // convergence test runs on the fp64 residual after the update
      if (S.rnorm <= S.ttol || S.rnorm < S.rdelta * S.rmax || i + 1 >= S.max_its) {
        S.hold = 1;
      } else {
        S.rmax = fmax(S.rmax, S.rnorm);
        S.beta = zrs;
        S.pcoef = S.beta / S.betaold;
        S.cg_i = i + 1;
      }
    } else if (S.rnorm <= S.ttol) {
      S.reason = FL_CONVERGED_RTOL;
      S.done = 1;
    } else if (i + 1 >= S.max_its) {
      S.reason = FL_DIVERGED_ITS;
      S.done = 1;
    } else {
      S.beta = zrs;
      S.pcoef = S.beta / S.betaold;
      S.cg_i = i + 1;
    }
  }
}

// Outer residual in fp64: r = b - A y; z = B r; and fp32 copies for the inner
// solve (r32 = z-scaled residual, z32 = B r32).  Partials ||Br||^2, ||Bb||^2, (Br).r
template <int G>
__global__ void k_outer_resid(SpArgs A, const double* __restrict__ b, const double* __restrict__ y,
                              const double* __restrict__ dinv, float* __restrict__ r32, float* __restrict__ z32,
                              float* __restrict__ d32, double* __restrict__ part, int nparts) {
  note_launch();
  __shared__ double red[kThreads / 32];
  const double piv = A.st->pivot;
  const int lane = threadIdx.x & 31, sub = lane & (G - 1);
  const int gpb = blockDim.x / G;
  const bool unprec = A.st->unprec;
  double zz = 0.0, bb = 0.0, zr = 0.0, rr = 0.0, bu = 0.0;
  for (int base = blockIdx.x * gpb; base < A.n; base += gridDim.x * gpb) {
    const int row = base + threadIdx.x / G;
    double s = 0.0;
    s = row_dot<G>(A.findrm, A.colm, A.val, y, row, sub, row < A.n);
    if (row < A.n && sub == 0) {
      if (A.ghost && A.ghost[row]) s = piv * y[row];
      const double ri = b[row] - s;
      const double zi = ri * dinv[row];
      const double bi = b[row] * dinv[row];
      r32[row] = (float)ri;
      z32[row] = (float)zi;
      d32[row] = 0.0f;
      zz += zi * zi;
      bb += bi * bi;
      zr += zi * ri;
      if (unprec) {
        rr += ri * ri;
        bu += b[row] * b[row];
      }
    }
  }
  zz = block_sum<kThreads>(zz, red);
  bb = block_sum<kThreads>(bb, red);
  zr = block_sum<kThreads>(zr, red);
  if (unprec) {
    rr = block_sum<kThreads>(rr, red);
    bu = block_sum<kThreads>(bu, red);
  }
  if (threadIdx.x == 0) {
    part[blockIdx.x] = zz;
    part[nparts + blockIdx.x] = bb;
    part[2 * nparts + blockIdx.x] = zr;
    if (unprec) {
      part[3 * nparts + blockIdx.x] = rr;
      part[4 * nparts + blockIdx.x] = bu;
    }
  }
}

// Reliable update, after y += d and the fp64 residual (k_outer_resid): the
// PETSc convergence test on the true preconditioned residual, then CG goes on
// from the same search direction with beta from the true residual.  The
// first call opens the solve (KSPConvergedDefault at iteration 0).
__global__ void k_rel_commit(KspState* st, const double* __restrict__ part, int nparts) {
  note_launch();
  __shared__ double red[kThreads / 32];
  const double zz = reduce_partials(part, nparts, red);
  const double bb = reduce_partials(part + nparts, nparts, red);
  const double zr = reduce_partials(part + 2 * nparts, nparts, red);
  const bool unprec = st->unprec;
  double rr = 0.0, bu = 0.0;
  if (unprec) {
    rr = reduce_partials(part + 3 * nparts, nparts, red);
    bu = reduce_partials(part + 4 * nparts, nparts, red);
  }
  if (threadIdx.x != 0) return;
  KspState& S = *st;
  const double rn = sqrt(unprec ? rr : zz);
  if (S.cg_i == 0 && S.outer == 0 && !S.hold) {
    S.snorm_b = sqrt(unprec ? bu : bb);
    S.its = 0;
    S.reason = 0;
    S.done = 0;
    converged_test(S, 0, rn);
    S.beta = zr;
    S.rmax = rn;
    return;
  }
  S.outer += 1;
  S.hold = 0;
  S.rnorm = rn;
  if (rn != rn) S.reason = FL_DIVERGED_NANORINF;
  else if (rn <= S.ttol) S.reason = rn < S.atol ? FL_CONVERGED_ATOL : FL_CONVERGED_RTOL;
  else if (rn >= S.dtol * S.rnorm0) S.reason = FL_DIVERGED_DTOL;
  else if (S.its >= S.max_its) S.reason = FL_DIVERGED_ITS;
  if (S.reason) {
    S.done = 1;
    return;
  }
  S.beta = zr;
  S.pcoef = zr / S.betaold;
  S.cg_i = S.its;
  S.rmax = rn;
}

__global__ void k_add_correction(int n, const float* __restrict__ d, double* __restrict__ y) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] += (double)d[i];
}

// ------------------------------------------------------------------ host --
struct Launch {
  unsigned grid;
  int nparts;
};

// Lanes per CSR row in the FP64 SpMV kernels.  FP64 throughput is scarce on
// this part, and each level of the in-group shuffle reduction costs a DADD on
// every lane, so short rows use two lanes.
static int group_for(const fl_mesh_t* m) {
  static int forced = [] {
    const char* e = getenv("FL_SPMV_LANES");
    return e ? atoi(e) : 0;
  }();
  if (forced == 1 || forced == 2 || forced == 4) return forced;
  const double avg = (double)m->nnz / (double)(m->N > 0 ? m->N : 1);
  if (avg > 24) return 4;
  return 2;
}

#define FL_SPMV32_DISPATCH(G, KERNEL, ...)                                          \
  do {                                                                             \
    if ((G) == 8) KERNEL<8><<<gsp32, kThreads, 0, s>>>(__VA_ARGS__);               \
    else KERNEL<4><<<gsp32, kThreads, 0, s>>>(__VA_ARGS__);                        \
  } while (0)

#define FL_SPMV_DISPATCH_S(G, STREAM, KERNEL, ...)                                  \
  do {                                                                             \
    if ((G) == 4) KERNEL<4><<<gsp, kThreads, 0, STREAM>>>(__VA_ARGS__);            \
    else if ((G) == 2) KERNEL<2><<<gsp, kThreads, 0, STREAM>>>(__VA_ARGS__);       \
    else KERNEL<1><<<gsp, kThreads, 0, STREAM>>>(__VA_ARGS__);                     \
  } while (0)
#define FL_SPMV_DISPATCH(G, KERNEL, ...) FL_SPMV_DISPATCH_S(G, s, KERNEL, __VA_ARGS__)

// Sliced-ELL pattern of the mesh, built once and cached on the workspace.
static int ensure_sell(fl_mesh_t* m, KrylovWork* W, cudaStream_t s) {
  if (W->sell_ready) return FL_OK;
  const int n = m->N;
  const int nsl = (n + kSlice - 1) / kSlice;
  FL_TRY(W->swidth.reserve(nsl + 1));
  FL_TRY(W->sptr.reserve(nsl + 1));
  k_sell_width<<<grid_for(nsl, kThreads), kThreads, 0, s>>>(m->findrm.p, n, nsl, W->swidth.p);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY(exclusive_scan_i32(W->swidth.p, W->sptr.p, nsl, s));
  int32_t len = 0;
  FL_TRY_CUDA(cudaMemcpyAsync(&len, W->sptr.p + nsl, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  FL_TRY(W->scol.reserve(len));
  FL_TRY(W->smap.reserve(len));
  FL_TRY(W->soff.reserve(len));
  DevBuf<int> wide;
  FL_TRY(wide.reserve(1));
  FL_TRY_CUDA(cudaMemsetAsync(wide.p, 0, sizeof(int), s));
  k_sell_fill<<<grid_for((int64_t)nsl * kSlice, kThreads), kThreads, 0, s>>>(m->findrm.p, m->colm.p, n, W->sptr.p,
                                                                             W->scol.p, W->smap.p, W->soff.p,
                                                                             wide.p);
  FL_TRY_CUDA(cudaGetLastError());
  int h_wide = 0;
  FL_TRY_CUDA(cudaMemcpyAsync(&h_wide, wide.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  W->sell16 = h_wide == 0;  // every column within 32767 of its row: 2-byte indices
  W->nslices = nsl;
  W->sell_len = len;
  W->sell_ready = true;
  return FL_OK;
}

// One FP64 CG iteration: three launches, no host interaction (capturable).
static void cg_iteration(int n, KspState* st, const SellArgs& SA, KrylovWork* W, unsigned gv, unsigned gsl, int np,
                         cudaStream_t s) {
  k_cg_p<<<gv, kThreads, 0, s>>>(n, st, W->z.p, W->p.p);
  k_cg_ap<<<gsl, kThreads, 0, s>>>(SA, W->sval.p, W->p.p, W->w2.p, W->part.p, W->ticket.p);
  k_cg_xr<<<gv, kThreads, 0, s>>>(n, st, W->p.p, W->w2.p, W->dinv.p, W->y.p, W->r.p, W->z.p, W->part.p + 2 * np,
                                   W->ticket.p + 1);
}

// One GMRES(restart) cycle with the restart decisions on the device
// (k_gmres_cycle_start with first = -1 takes the first-cycle flag from the
// state, k_gmres_cycle_end applies the iteration limit and clears the zero
// guess); every launch returns at once when the solve has converged, so
// cycles may be replayed past convergence.  No host interaction (capturable).
static void gmres_cycle_launch(int G, const SpArgs& A, KrylovWork* W, int n, int restart, unsigned gsp,
                               unsigned gv, cudaStream_t s) {
  KspState* st = A.st;
  const int64_t ld = n;
  double* V = W->V.p;
  double* U = W->w.p;  // the unnormalised next basis vector
  FL_SPMV_DISPATCH(G, k_init_resid, A, W->b.p, W->y.p, W->dinv.p, W->r.p, U, W->part.p, (int)gsp);
  k_gmres_cycle_start<<<1, kThreads, 0, s>>>(st, W->part.p, (int)gsp, -1);
  for (int it = 0; it < restart; ++it) {
    FL_SPMV_DISPATCH(G, k_gmres_arnoldi, A, W->dinv.p, V, U, ld, it, W->part.p, W->ticket.p + 2);
    k_gmres_orth<<<gv, kThreads, 0, s>>>(n, st, V, U, ld, it, restart, W->part.p, W->ticket.p + 3);
  }
  k_gmres_backsolve<<<1, 32, 0, s>>>(st, restart);
  k_gmres_update_x<<<gv, kThreads, 0, s>>>(n, st, V, ld, W->y.p);
  k_gmres_cycle_end<<<1, 32, 0, s>>>(st);
}

int solve(fl_mesh_t* m, const fl_solver_opts* o, const double* val, const uint8_t* ghost, const double* rhs,
          double* x, fl_solve_report* rep, cudaStream_t s) {
  FL_CHECK_ARG(m && o && val && rhs && x && rep, "null argument");
  FL_CHECK_ARG(o->ksp_type == 0 || o->ksp_type == 1, "ksp_type must be 0 (cg) or 1 (gmres)");
  FL_CHECK_ARG(o->max_its >= 0, "max_its");
  const int restart = o->restart > 0 ? o->restart : 30;
  FL_CHECK_ARG(restart <= kMaxRestart, "gmres restart above 64");
  FL_CHECK_ARG(o->precision == 0 || o->ksp_type == 0, "mixed precision is a CG refinement");
  FL_CHECK_ARG(o->precision >= 0 && o->precision <= 2, "precision 0 (fp64), 1 or 2 (mixed)");
  FL_CHECK_ARG(o->norm_type == 0 || o->norm_type == 1, "norm_type 0 (preconditioned) or 1 (unpreconditioned)");
  FL_CHECK_ARG(o->norm_type == 0 || o->ksp_type == 0,
               "the unpreconditioned norm needs CG (left-preconditioned GMRES tests the preconditioned norm)");
  KrylovWork* W = work_of(m);
  if (!W) return FL_ERR_NOMEM;
  const int n = m->N;
  const int G = group_for(m);
  const unsigned gsp = grid_for((int64_t)n * G, kThreads, 8);
  const unsigned gv = grid_for(n, kThreads, 4);
  const int np = (int)std::max(gsp, gv);
  FL_TRY(W->b.reserve(n));
  FL_TRY(W->y.reserve(n));
  FL_TRY(W->r.reserve(n));
  FL_TRY(W->z.reserve(n));
  FL_TRY(W->p.reserve(n));
  FL_TRY(W->w.reserve(n));
  FL_TRY(W->dinv.reserve(n));
  FL_TRY(W->part.reserve((size_t)np * (kMaxRestart + 2)));
  FL_TRY(W->st.reserve(1));
  if (!W->pin) FL_TRY_CUDA(cudaMallocHost(&W->pin, sizeof(KrylovWork::HostPin)));
  // the previous solve on this workspace ended with a synchronisation, so
  // the pinned buffer is free
  KspState& h = W->pin->st;
  std::memset(&h, 0, offsetof(KspState, grs));
  W->pin->fault = 0;
  h.rtol = o->rtol;
  h.atol = o->atol;
  h.dtol = o->dtol > 0 ? o->dtol : 1e5;
  h.max_its = o->max_its;
  h.guess_zero = o->start_from_zero ? 1 : 0;
  h.unprec = o->norm_type == 1 ? 1 : 0;
  h.gm_first = 1;
  // the scalars only: the GMRES arrays behind them are written before they
  // are read in every cycle
  FL_TRY_CUDA(cudaMemcpyAsync(W->st.p, &h, offsetof(KspState, grs), cudaMemcpyHostToDevice, s));
  KspState* st = W->st.p;
  SpArgs A{n, m->findrm.p, m->colm.p, val, ghost, st};

  // Jacobi diagonal and ghost pivot
  // retire tickets: [0..3] the Krylov kernels, [4] the diagonal pass, [5] the true residual
  FL_TRY(W->ticket.reserve(6));
  FL_TRY_CUDA(cudaMemsetAsync(W->ticket.p, 0, sizeof(unsigned) * 6, s));
  k_diag<<<gv, kThreads, 0, s>>>(A, m->centrm.p, W->dinv.p, W->part.p, W->part.p + np, W->ticket.p + 4);
  const bool mixed = o->precision != 0;
  if (mixed) FL_TRY(W->dinv32.reserve(n));
  FL_SPMV_DISPATCH(G, k_lift, A, rhs, x, h.guess_zero, W->b.p, W->y.p, W->dinv.p, mixed ? W->dinv32.p : nullptr);
  FL_TRY_CUDA(cudaGetLastError());

  int outer = 0;
  const int chunk = 16;
  // FP64 GMRES in one cooperative launch: schedule 2, or 0 up to
  // FL_PERSIST_MAX_ROWS rows; one block per group of kThreads / G rows, at
  // most one per SM, and only when that many blocks can be co-resident
  bool persistent = false;
  int pnb = 0, npass = 0, ppg = 8;
  size_t psmem = 0;
  if (o->ksp_type == 1 && !mixed && (o->schedule == 2 || (o->schedule == 0 && n <= FL_PERSIST_MAX_ROWS))) {
    const int sms = num_sms();
    ppg = (n + kThreads / 8 - 1) / (kThreads / 8) <= sms ? 8 : (n + kThreads / 4 - 1) / (kThreads / 4) <= sms ? 4 : 2;
    const int rows_per_pass = kThreads / ppg;
    const int groups = (n + rows_per_pass - 1) / rows_per_pass;
    // launch shape of this (lanes per row, rows, restart), worked out once
    // per process (occupancy queries and the shared-memory attribute)
    struct Shape {
      int pg, groups, restart, npass, pnb, ok;
      size_t smem;
    };
    static std::vector<Shape> shapes;
    static std::mutex shapes_mu;
    std::lock_guard<std::mutex> lock(shapes_mu);
    const Shape* hit = nullptr;
    for (const Shape& c : shapes)
      if (c.pg == ppg && c.groups == groups && c.restart == restart) hit = &c;
    if (!hit) {
      const void* fn = ppg == 8 ? (const void*)k_gmres_persistent<8>
                     : ppg == 4 ? (const void*)k_gmres_persistent<4> : (const void*)k_gmres_persistent<2>;
      Shape c{ppg, groups, restart, 0, 0, 0, 0};
      int per_sm = 0;
      FL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, 0));
      const int cap = std::max(1, per_sm) * sms;
      c.npass = (groups + cap - 1) / cap;
      c.pnb = (groups + c.npass - 1) / c.npass;
      c.smem = persist_smem_bytes(restart, c.npass, ppg);
      cudaFuncAttributes fa;
      FL_TRY_CUDA(cudaFuncGetAttributes(&fa, fn));
      int dev = 0, optin = 0;
      FL_TRY_CUDA(cudaGetDevice(&dev));
      FL_TRY_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
      if (fa.sharedSizeBytes + c.smem <= (size_t)optin) {
        // the attribute only grows, so a smaller shape cached earlier stays valid
        int cur = 0;
        cudaFuncAttributes fb;
        FL_TRY_CUDA(cudaFuncGetAttributes(&fb, fn));
        cur = fb.maxDynamicSharedSizeBytes;
        if ((int)c.smem > cur) FL_TRY_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)c.smem));
        FL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, c.smem));
        c.ok = (int64_t)per_sm * sms >= c.pnb ? 1 : 0;
      }
      shapes.push_back(c);
      hit = &shapes.back();
    }
    persistent = hit->ok != 0;
    npass = hit->npass;
    pnb = hit->pnb;
    psmem = hit->smem;
    if (persistent) FL_TRY(W->part.reserve((size_t)std::max(np, pnb) * (kMaxRestart + 3)));
  }
  FL_TRY(ensure_sell(m, W, s));
  SellArgs SA{n, W->sptr.p, W->scol.p, ghost, st, W->sell16 ? W->soff.p : nullptr};
  const unsigned gsl = grid_for(n, kThreads, 8);
  if (!mixed && o->ksp_type == 0) {
    FL_SPMV_DISPATCH(G, k_init_resid, A, W->b.p, W->y.p, W->dinv.p, W->r.p, W->z.p, W->part.p, (int)gsp);
    k_cg_start<<<1, kThreads, 0, s>>>(st, W->part.p, (int)gsp);
    FL_TRY_CUDA(cudaGetLastError());
    FL_TRY(W->w2.reserve(n));
    FL_TRY(W->ticket.reserve(4));
    FL_TRY(W->sval.reserve(W->sell_len));
    FL_TRY_CUDA(cudaMemsetAsync(W->ticket.p, 0, sizeof(unsigned) * 4, s));
    k_sell_values<<<grid_for(W->sell_len, kThreads), kThreads, 0, s>>>(W->sell_len, W->smap.p, val, W->sval.p,
                                                                         nullptr);
    k_cg_open<<<1, 32, 0, s>>>(st);
    FL_TRY_CUDA(cudaGetLastError());
    // chunks of `chunk` iterations replayed as one graph until the device
    // reports convergence or the iteration limit (iterations past the end
    // of the solve return at once)
    IterGraph gr{W, s};
    const std::vector<uintptr_t> key{
        (uintptr_t)n,        (uintptr_t)gv,       (uintptr_t)gsl,      (uintptr_t)np,      (uintptr_t)ghost,
        (uintptr_t)st,       (uintptr_t)SA.sptr,  (uintptr_t)SA.scol,  (uintptr_t)SA.soff, (uintptr_t)W->z.p,
        (uintptr_t)W->p.p,   (uintptr_t)W->w2.p,  (uintptr_t)W->part.p, (uintptr_t)W->ticket.p,
        (uintptr_t)W->dinv.p, (uintptr_t)W->y.p,  (uintptr_t)W->r.p,   (uintptr_t)W->sval.p};
    FL_TRY(gr.build_cached(W->g_cg, key, [&](cudaStream_t c) {
      for (int k = 0; k < chunk; ++k) cg_iteration(n, st, SA, W, gv, gsl, np, c);
    }));
    // with the unpreconditioned norm a convergence is confirmed on the
    // recomputed residual (at most a few replacements; each normally passes)
    for (int confirm = 0; confirm < (o->norm_type == 1 ? 4 : 1); ++confirm) {
      for (int i = 0; i < o->max_its; i += chunk) {
        FL_TRY(gr.launch());
        int done = 0;
        FL_TRY_CUDA(cudaMemcpyAsync(&done, &st->done, sizeof(int), cudaMemcpyDeviceToHost, W->cs));
        FL_TRY_CUDA(cudaStreamSynchronize(W->cs));
        if (done) break;
      }
      if (o->norm_type != 1) break;
      int hr[2] = {0, 0};
      FL_TRY_CUDA(cudaMemcpyAsync(hr, &st->reason, sizeof(int) * 2, cudaMemcpyDeviceToHost, W->cs));
      FL_TRY_CUDA(cudaStreamSynchronize(W->cs));
      if (hr[0] != FL_CONVERGED_RTOL) break;
      const cudaStream_t c = W->cs;
      k_cg_reopen<<<1, 32, 0, c>>>(st);
      FL_SPMV_DISPATCH_S(G, c, k_init_resid, A, W->b.p, W->y.p, W->dinv.p, W->r.p, W->z.p, W->part.p, (int)gsp);
      k_cg_confirm<<<1, kThreads, 0, c>>>(st, W->part.p, (int)gsp);
      FL_TRY_CUDA(cudaGetLastError());
      int done = 0;
      FL_TRY_CUDA(cudaMemcpyAsync(&done, &st->done, sizeof(int), cudaMemcpyDeviceToHost, c));
      FL_TRY_CUDA(cudaStreamSynchronize(c));
      if (done) break;
    }
    FL_TRY(gr.join());
    FL_TRY_CUDA(cudaGetLastError());
  } else if (!mixed && persistent) {
    // GMRES(restart) in one cooperative launch (k_gmres_persistent)
    FL_TRY(W->ticket.reserve(4));
    FL_TRY_CUDA(cudaMemsetAsync(W->ticket.p, 0, sizeof(unsigned) * 4, s));
    const WaitTest& wt = wait_test();
    PersistArgs P{A,      W->dinv.p, W->b.p, W->y.p, W->w.p, reinterpret_cast<float2*>(W->part.p),
                  reinterpret_cast<unsigned long long*>(W->ticket.p), restart, npass, wt.withhold,
                  wt.wait_ms > 0.0 ? (unsigned long long)(wt.wait_ms * 1e6) : kBarrierWaitNs};
    void* args[] = {&P};
    const void* fn = ppg == 8 ? (const void*)k_gmres_persistent<8>
                   : ppg == 4 ? (const void*)k_gmres_persistent<4> : (const void*)k_gmres_persistent<2>;
    FL_TRY_CUDA(cudaLaunchCooperativeKernel(fn, dim3(pnb), dim3(kThreads), args, psmem, s));
    FL_TRY_CUDA(cudaMemcpyAsync(&W->pin->fault, W->ticket.p + 2, sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, s));
  } else if (!mixed) {
    // GMRES(restart): one cycle with the restarts decided on the device,
    // captured as a graph and replayed until the device reports the end of
    // the solve (each cycle either ends it or advances the iteration count,
    // and the iteration limit ends it)
    FL_TRY(W->V.reserve((size_t)(restart + 1) * n));
    FL_TRY(W->ticket.reserve(4));
    FL_TRY_CUDA(cudaMemsetAsync(W->ticket.p, 0, sizeof(unsigned) * 4, s));
    IterGraph gr{W, s};
    const std::vector<uintptr_t> key{
        (uintptr_t)n,       (uintptr_t)G,        (uintptr_t)gsp,       (uintptr_t)gv,       (uintptr_t)restart,
        (uintptr_t)val,     (uintptr_t)ghost,    (uintptr_t)m->findrm.p, (uintptr_t)m->colm.p, (uintptr_t)st,
        (uintptr_t)W->b.p,  (uintptr_t)W->y.p,   (uintptr_t)W->r.p,    (uintptr_t)W->dinv.p, (uintptr_t)W->V.p,
        (uintptr_t)W->part.p, (uintptr_t)W->ticket.p, (uintptr_t)W->w.p};
    FL_TRY(gr.build_cached(W->g_gmres, key,
                           [&](cudaStream_t c) { gmres_cycle_launch(G, A, W, n, restart, gsp, gv, c); }));
    for (int cycle = 0; cycle <= o->max_its; ++cycle) {
      FL_TRY(gr.launch());
      int done = 0;
      FL_TRY_CUDA(cudaMemcpyAsync(&done, &st->done, sizeof(int), cudaMemcpyDeviceToHost, W->cs));
      FL_TRY_CUDA(cudaStreamSynchronize(W->cs));
      if (done) break;
    }
    FL_TRY(gr.join());
    FL_TRY_CUDA(cudaGetLastError());
  } else {
    // Mixed precision: fp32 inner CG (rtol inner_rtol) inside fp64 refinement
    FL_TRY(W->r32.reserve(n));
    FL_TRY(W->z32.reserve(n));
    FL_TRY(W->p32.reserve(n));
    FL_TRY(W->w32.reserve(n));
    FL_TRY(W->d32.reserve(n));
    FL_TRY(W->ticket.reserve(4));
    FL_TRY_CUDA(cudaMemsetAsync(W->ticket.p, 0, sizeof(unsigned) * 4, s));
    FL_TRY(W->sval32.reserve(W->sell_len));
    k_sell_values<<<grid_for(W->sell_len, kThreads), kThreads, 0, s>>>(W->sell_len, W->smap.p, val, nullptr,
                                                                         W->sval32.p);
    FL_TRY_CUDA(cudaGetLastError());
    KspState hs;
    FL_TRY_CUDA(cudaMemcpyAsync(&hs, st, sizeof(KspState), cudaMemcpyDeviceToHost, s));
    FL_TRY_CUDA(cudaStreamSynchronize(s));
    const float piv32 = (float)hs.pivot;
    const double inner_rtol = o->inner_rtol > 0 ? o->inner_rtol : 1e-5;
    double rnorm0 = 0.0, ttol = 0.0;
    int total_inner = 0, reason = 0;
    if (o->precision == 2) {
      // fp32 CG with reliable updates (Sleijpen and van der Vorst, 1996): the
      // fp32 recurrence runs without restarts; whenever its residual has
      // dropped by rdelta since the last update, or claims convergence, the
      // correction is added to the fp64 solution, the fp64 residual replaces
      // the recurrence residual and the convergence test runs on it.
      hs.rel = 1;
      hs.hold = 0;
      hs.outer = 0;
      hs.cg_i = 0;
      hs.rdelta = 0.1;
      hs.rmax = 0.0;
      FL_TRY_CUDA(cudaMemcpyAsync(st, &hs, sizeof(KspState), cudaMemcpyHostToDevice, s));
      auto update = [&]() {
        FL_SPMV_DISPATCH(G, k_outer_resid, A, W->b.p, W->y.p, W->dinv.p, W->r32.p, W->z32.p, W->d32.p,
                         W->part.p, (int)gsp);
        k_rel_commit<<<1, kThreads, 0, s>>>(st, W->part.p, (int)gsp);
      };
      update();
      FL_TRY_CUDA(cudaGetLastError());
      IterGraph gr{W, s};
      FL_TRY(gr.build([&](cudaStream_t c) {
        for (int k = 0; k < chunk; ++k) {
          k_cg32_p<<<gv, kThreads, 0, c>>>(n, st, W->z32.p, W->p32.p);
          k_cg32_ap<<<gsl, kThreads, 0, c>>>(SA, W->sval32.p, piv32, W->p32.p, W->w32.p, W->part.p,
                                              W->ticket.p);
          k_cg32_xr<<<gv, kThreads, 0, c>>>(n, st, W->p32.p, W->w32.p, W->dinv32.p, W->d32.p, W->r32.p,
                                             W->z32.p, W->part.p + 2 * np, W->ticket.p + 1);
        }
      }));
      const cudaStream_t c = W->cs;
      auto update_c = [&]() {
        FL_SPMV_DISPATCH_S(G, c, k_outer_resid, A, W->b.p, W->y.p, W->dinv.p, W->r32.p, W->z32.p, W->d32.p,
                           W->part.p, (int)gsp);
        k_rel_commit<<<1, kThreads, 0, c>>>(st, W->part.p, (int)gsp);
      };
      for (int i = 0; i < 1000000; i += chunk) {
        FL_TRY(gr.launch());
        KspState h2;
        FL_TRY_CUDA(cudaMemcpyAsync(&h2.its, &st->its, sizeof(int) * 4, cudaMemcpyDeviceToHost, c));
        FL_TRY_CUDA(cudaMemcpyAsync(&h2.hold, &st->hold, sizeof(int), cudaMemcpyDeviceToHost, c));
        FL_TRY_CUDA(cudaStreamSynchronize(c));
        if (h2.done) break;
        if (h2.hold) {
          k_add_correction<<<gv, kThreads, 0, c>>>(n, W->d32.p, W->y.p);
          update_c();
          FL_TRY_CUDA(cudaGetLastError());
        }
      }
      FL_TRY(gr.join());
      // a solve stopped inside the fp32 recurrence keeps its last correction
      k_add_correction<<<gv, kThreads, 0, s>>>(n, W->d32.p, W->y.p);
      FL_TRY_CUDA(cudaMemcpyAsync(&hs, st, sizeof(KspState), cudaMemcpyDeviceToHost, s));
      FL_TRY_CUDA(cudaStreamSynchronize(s));
      hs.rel = 0;
      FL_TRY_CUDA(cudaMemcpyAsync(&st->rel, &hs.rel, sizeof(int), cudaMemcpyHostToDevice, s));
    }
    const int rel_updates = hs.outer;
    for (outer = 0; o->precision == 1 && outer < 1000; ++outer) {
      FL_SPMV_DISPATCH(G, k_outer_resid, A, W->b.p, W->y.p, W->dinv.p, W->r32.p, W->z32.p, W->d32.p, W->part.p,
                       (int)gsp);
      k_cg_start<<<1, kThreads, 0, s>>>(st, W->part.p, (int)gsp);
      FL_TRY_CUDA(cudaGetLastError());
      FL_TRY_CUDA(cudaMemcpyAsync(&hs, st, sizeof(KspState), cudaMemcpyDeviceToHost, s));
      FL_TRY_CUDA(cudaStreamSynchronize(s));
      const double rn = hs.rnorm;
      if (outer == 0) {
        rnorm0 = hs.rnorm0;
        ttol = hs.ttol;
      }
      if (rn != rn) { reason = FL_DIVERGED_NANORINF; break; }
      if (rn <= ttol) { reason = rn < o->atol ? FL_CONVERGED_ATOL : FL_CONVERGED_RTOL; break; }
      if (total_inner >= o->max_its) { reason = FL_DIVERGED_ITS; break; }
      // inner solve B A d = B r in fp32 from d = 0 to inner_rtol * ||B r||
      // (the inner test is on the preconditioned fp32 residual whichever
      // norm the outer test uses)
      hs.ttol = inner_rtol * hs.znorm;
      hs.done = 0;
      hs.reason = 0;
      hs.dpi = 0.0;
      hs.its = 0;
      hs.pcoef = 0.0;
      hs.cg_i = 0;
      hs.max_its = o->max_its - total_inner;
      FL_TRY_CUDA(cudaMemcpyAsync(st, &hs, sizeof(KspState), cudaMemcpyHostToDevice, s));
      int inner = 0;
      for (int i = 0; i < hs.max_its; ++i) {
        k_cg32_p<<<gv, kThreads, 0, s>>>(n, st, W->z32.p, W->p32.p);
        k_cg32_ap<<<gsl, kThreads, 0, s>>>(SA, W->sval32.p, piv32, W->p32.p, W->w32.p, W->part.p, W->ticket.p);
        k_cg32_xr<<<gv, kThreads, 0, s>>>(n, st, W->p32.p, W->w32.p, W->dinv32.p, W->d32.p, W->r32.p,
                                           W->z32.p, W->part.p + 2 * np, W->ticket.p + 1);
        if ((i + 1) % chunk == 0 || i + 1 == hs.max_its) {
          FL_TRY_CUDA(cudaGetLastError());
          KspState h2;
          FL_TRY_CUDA(cudaMemcpyAsync(&h2.its, &st->its, sizeof(int) * 4, cudaMemcpyDeviceToHost, s));
          FL_TRY_CUDA(cudaStreamSynchronize(s));
          inner = h2.its;
          if (h2.done) break;
        }
      }
      total_inner += inner;
      k_add_correction<<<gv, kThreads, 0, s>>>(n, W->d32.p, W->y.p);
      FL_TRY_CUDA(cudaGetLastError());
    }
    if (o->precision == 2) outer = rel_updates;
    if (o->precision == 1) {
      // report in the outer terms
      hs.its = total_inner;
      hs.reason = reason;
      hs.rnorm0 = rnorm0;
      FL_TRY_CUDA(cudaMemcpyAsync(&st->its, &hs.its, sizeof(int), cudaMemcpyHostToDevice, s));
      FL_TRY_CUDA(cudaMemcpyAsync(&st->reason, &hs.reason, sizeof(int), cudaMemcpyHostToDevice, s));
      FL_TRY_CUDA(cudaMemcpyAsync(&st->rnorm0, &hs.rnorm0, sizeof(double), cudaMemcpyHostToDevice, s));
    }
  }
  FL_SPMV_DISPATCH(G, k_true_resid, A, W->b.p, W->y.p, W->part.p, (int)gsp, rhs, x, W->ticket.p + 5);
  FL_TRY_CUDA(cudaGetLastError());
  KspState& hs = W->pin->st;
  FL_TRY_CUDA(cudaMemcpyAsync(&hs, st, offsetof(KspState, grs), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  if (W->pin->fault) {
    set_error("a bounded device wait ran out: a grid barrier of the cooperative GMRES solve");
    return FL_ERR_TIMEOUT;
  }
  rep->iterations = hs.its;
  rep->reason = hs.reason ? hs.reason : (o->max_its == 0 ? FL_DIVERGED_ITS : 0);
  rep->final_rnorm = hs.rnorm;
  rep->rnorm0 = hs.rnorm0;
  rep->true_rel_residual = hs.b2 > 0 ? sqrt(hs.true_r2 / hs.b2) : sqrt(hs.true_r2);
  rep->outer_iterations = outer;
  rep->pad = 0;
  return FL_OK;
}

// ------------------------------------------------- batched / graph CG --
__global__ void k_state_init(KspState* st, double rtol, double atol, double dtol, int max_its, int guess_zero,
                             int unprec) {
  note_launch();
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  KspState& S = *st;
  S.unprec = unprec;
  S.rtol = rtol;
  S.atol = atol;
  S.dtol = dtol;
  S.max_its = max_its;
  S.guess_zero = guess_zero;
  S.rnorm0 = S.ttol = S.snorm_b = S.rnorm = 0.0;
  S.its = S.reason = S.done = 0;
  S.cg_i = 0;
  S.beta = S.betaold = S.dpi = S.dpiold = S.alpha = S.pcoef = S.dpi_next = 0.0;
  S.true_r2 = S.b2 = 0.0;
  S.it = S.hapend = S.live = 0;
  S.gm_first = 1;
  S.tt = 0.0;
}

// done flags of several solves gathered into one array (polled by the host)
__global__ void k_gather_done(KspState* const* sts, int n, int* out) {
  note_launch();
  for (int i = threadIdx.x; i < n; i += blockDim.x) out[i] = sts[i]->done;
}

int cg_prepare(CgPlan& P, fl_mesh_t* m, const fl_solver_opts* o, const double* val, const uint8_t* ghost,
               const double* rhs, double* x, cudaStream_t s) {
  FL_CHECK_ARG(m && o && val && rhs && x, "null argument");
  FL_CHECK_ARG((o->ksp_type == 0 || o->ksp_type == 1) && o->precision == 0,
               "graph-batched solves are FP64 CG or GMRES");
  FL_CHECK_ARG(o->norm_type == 0 || (o->norm_type == 1 && o->ksp_type == 0),
               "norm_type 0, or 1 (unpreconditioned) with CG");
  FL_CHECK_ARG(o->max_its >= 0, "max_its");
  const int restart = o->restart > 0 ? o->restart : 30;
  FL_CHECK_ARG(restart <= kMaxRestart, "gmres restart above 64");
  KrylovWork* M = work_of(m);  // pattern owner
  if (!M) return FL_ERR_NOMEM;
  FL_TRY(ensure_sell(m, M, s));
  if (!P.W) P.W = new KrylovWork();
  KrylovWork* W = P.W;
  const int n = m->N;
  P.m = m;
  P.o = *o;
  P.val = val;
  P.ghost = ghost;
  P.rhs = rhs;
  P.x = x;
  P.n = n;
  P.G = group_for(m);
  P.gsp = grid_for((int64_t)n * P.G, kThreads, 8);
  P.gv = grid_for(n, kThreads, 4);
  P.gsl = grid_for(n, kThreads, 8);
  P.np = (int)std::max(P.gsp, P.gv);
  P.ksp = o->ksp_type;
  P.restart = restart;
  if (P.ksp == 1) {
    FL_TRY(W->V.reserve((size_t)(restart + 1) * n));
    FL_TRY(W->w.reserve(n));
  }
  FL_TRY(W->b.reserve(n));
  FL_TRY(W->y.reserve(n));
  FL_TRY(W->r.reserve(n));
  FL_TRY(W->z.reserve(n));
  FL_TRY(W->p.reserve(n));
  FL_TRY(W->w2.reserve(n));
  FL_TRY(W->dinv.reserve(n));
  FL_TRY(W->part.reserve((size_t)P.np * (kMaxRestart + 2)));
  FL_TRY(W->st.reserve(1));
  FL_TRY(W->ticket.reserve(6));
  FL_TRY(W->sval.reserve(M->sell_len));
  P.sell_len = M->sell_len;
  P.smap = M->smap.p;
  P.SA = SellArgs{n, M->sptr.p, M->scol.p, ghost, W->st.p, M->sell16 ? M->soff.p : nullptr};
  P.A = SpArgs{n, m->findrm.p, m->colm.p, val, ghost, W->st.p};
  return FL_OK;
}

// Everything before the first iteration, as device work only (capturable).
void cg_setup_launch(CgPlan& P, cudaStream_t s) {
  KrylovWork* W = P.W;
  KspState* st = W->st.p;
  const int G = P.G;
  const unsigned gsp = P.gsp;
  k_state_init<<<1, 32, 0, s>>>(st, P.o.rtol, P.o.atol, P.o.dtol > 0 ? P.o.dtol : 1e5, P.o.max_its,
                                 P.o.start_from_zero ? 1 : 0, P.o.norm_type == 1 ? 1 : 0);
  cudaMemsetAsync(W->ticket.p, 0, sizeof(unsigned) * 6, s);
  k_diag<<<P.gv, kThreads, 0, s>>>(P.A, P.m->centrm.p, W->dinv.p, W->part.p, W->part.p + P.np, W->ticket.p + 4);
  FL_SPMV_DISPATCH(G, k_lift, P.A, P.rhs, P.x, P.o.start_from_zero ? 1 : 0, W->b.p, W->y.p, W->dinv.p, nullptr);
  if (P.ksp == 1) return;  // GMRES: the first cycle computes the initial residual
  FL_SPMV_DISPATCH(G, k_init_resid, P.A, W->b.p, W->y.p, W->dinv.p, W->r.p, W->z.p, W->part.p, (int)gsp);
  k_cg_start<<<1, kThreads, 0, s>>>(st, W->part.p, (int)gsp);
  cudaMemsetAsync(W->p.p, 0, sizeof(double) * P.n, s);
  k_sell_values<<<grid_for(P.sell_len, kThreads), kThreads, 0, s>>>(P.sell_len, P.smap, P.val, W->sval.p, nullptr);
  k_cg_open<<<1, 32, 0, s>>>(st);
}

// One GMRES(restart) cycle of a batched plan.
static void gmres_cycle(CgPlan& P, cudaStream_t s) {
  gmres_cycle_launch(P.G, P.A, P.W, P.n, P.restart, P.gsp, P.gv, s);
}

void cg_iterate(CgPlan& P, cudaStream_t s) {
  if (P.ksp == 1) gmres_cycle(P, s);
  else cg_iteration(P.n, P.W->st.p, P.SA, P.W, P.gv, P.gsl, P.np, s);
}

void cg_finish_launch(CgPlan& P, cudaStream_t s) {
  KrylovWork* W = P.W;
  const int G = P.G;
  const unsigned gsp = P.gsp;
  FL_SPMV_DISPATCH(G, k_true_resid, P.A, W->b.p, W->y.p, W->part.p, (int)gsp, P.rhs, P.x, W->ticket.p + 5);
}

int cg_report(CgPlan& P, fl_solve_report* rep, cudaStream_t s) {
  KspState hs;
  FL_TRY_CUDA(cudaMemcpyAsync(&hs, P.W->st.p, sizeof(KspState), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  rep->iterations = hs.its;
  rep->reason = hs.reason ? hs.reason : FL_DIVERGED_ITS;
  rep->final_rnorm = hs.rnorm;
  rep->rnorm0 = hs.rnorm0;
  rep->true_rel_residual = hs.b2 > 0 ? sqrt(hs.true_r2 / hs.b2) : sqrt(hs.true_r2);
  rep->outer_iterations = 0;
  rep->pad = 0;
  return FL_OK;
}

void cg_release(CgPlan& P) {
  delete P.W;
  P.W = nullptr;
}

KspState* cg_state(CgPlan& P) { return P.W->st.p; }

void gather_done(KspState* const* d_states, int n, int* d_out, cudaStream_t s) {
  k_gather_done<<<1, 128, 0, s>>>(d_states, n, d_out);
}

// Cached workspace per mesh handle.
struct WorkRegistry {
  std::vector<std::pair<fl_mesh_t*, KrylovWork*>> v;
} g_work;

static KrylovWork* work_of(fl_mesh_t* m) {
  for (auto& e : g_work.v)
    if (e.first == m) return e.second;
  KrylovWork* w = new KrylovWork();
  g_work.v.push_back({m, w});
  return w;
}

void release_krylov_work(fl_mesh_t* m) {
  for (size_t i = 0; i < g_work.v.size(); ++i)
    if (g_work.v[i].first == m) {
      delete g_work.v[i].second;
      g_work.v.erase(g_work.v.begin() + i);
      return;
    }
}

template <int G>
__global__ void k_spmv_plain(SpArgs A, const double* __restrict__ x, double* __restrict__ y) {
  note_launch();
  const int lane = threadIdx.x & 31, sub = lane & (G - 1);
  const int gpb = blockDim.x / G;
  for (int base = blockIdx.x * gpb; base < A.n; base += gridDim.x * gpb) {
    const int row = base + threadIdx.x / G;
    double s = 0.0;
    s = row_dot<G>(A.findrm, A.colm, A.val, x, row, sub, row < A.n);
    if (row < A.n && sub == 0) y[row] = s;
  }
}

int csr_mult(fl_mesh_t* m, const double* val, const double* x, double* y, cudaStream_t s) {
  const int G = group_for(m);
  const unsigned gsp = grid_for((int64_t)m->N * G, kThreads, 8);
  SpArgs A{m->N, m->findrm.p, m->colm.p, val, nullptr, nullptr};
  FL_SPMV_DISPATCH(G, k_spmv_plain, A, x, y);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

}  // namespace fl

using namespace fl;

extern "C" int fl_dev_petsc_solve(fl_mesh m, const fl_solver_opts* o, const double* val, const uint8_t* inactive,
                                  const double* rhs, double* x, fl_solve_report* rep, void* stream) {
  FL_CHECK_ARG(m, "null mesh");
  cudaStream_t s = stream ? (cudaStream_t)stream : m->stream;
  return solve(m, o, val, inactive, rhs, x, rep, s);
}

namespace fl {
// t_new = t + dt delta (the acceleration-form update of solve_field_equation_cg),
// the product rounded before the sum as the separate statement rounds it
// (no FMA contraction)
__global__ void k_field_update(int n, const double* __restrict__ t, double dt, const double* __restrict__ d,
                               double* __restrict__ out) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = __dadd_rn(t ? t[i] : 0.0, __dmul_rn(dt, d[i]));
}
}  // namespace fl

extern "C" int fl_dev_solve_field_equation_cg(fl_mesh m, const fl_advdif_params* p, const fl_fields* f, int32_t nb,
                                              const int32_t* bc_nodes, int32_t index_base, const double* bc_values,
                                              const fl_solver_opts* o, double* val, double* rhs, uint8_t* inactive,
                                              double* delta, double* t_new, fl_solve_report* rep, void* stream) {
  FL_CHECK_ARG(m && p && f && o && val && rhs && inactive && delta && t_new && rep, "null argument");
  FL_CHECK_ARG(nb >= 0 && (nb == 0 || (bc_nodes && bc_values)), "boundary node list");
  cudaStream_t s = stream ? (cudaStream_t)stream : m->stream;
  // assemble (M + theta dt (A + K)) delta = rhs
  FL_TRY(assemble(m, p, f, val, rhs, s, nullptr));
  // strong Dirichlet conditions in rate-of-change form: rhs = (g - t) / dt
  FL_TRY_CUDA(cudaMemsetAsync(inactive, 0, (size_t)m->N, s));
  FL_TRY(dirichlet_launch(m, nb, bc_nodes, index_base, bc_values, f->t, p->dt, rhs, inactive, s));
  // petsc_solve(delta_t, ...) from zero change
  FL_TRY_CUDA(cudaMemsetAsync(delta, 0, sizeof(double) * (size_t)m->N, s));
  FL_TRY(solve(m, o, val, inactive, rhs, delta, rep, s));
  k_field_update<<<grid_for(m->N, kThreads, 4), kThreads, 0, s>>>(m->N, f->t, p->dt, delta, t_new);
  FL_TRY_CUDA(cudaGetLastError());
  // pattern misses and out-of-range boundary nodes, reported once for the step
  return check_err(m->err.p, s, "assembly or Dirichlet conditions of solve_field_equation_cg");
}

extern "C" int fl_gpu_petsc_solve(fl_mesh m, const fl_solver_opts* o, const double* val, const uint8_t* inactive,
                                  const double* rhs, double* x, fl_solve_report* rep) {
  FL_CHECK_ARG(m && o && val && rhs && x && rep, "null argument");
  cudaStream_t s = m->stream;
  FL_TRY(m->st_val.reserve(m->nnz));
  FL_TRY(m->st_rhs.reserve(m->N));
  FL_TRY(m->st_x.reserve(m->N));
  FL_TRY_CUDA(cudaMemcpyAsync(m->st_val.p, val, sizeof(double) * m->nnz, cudaMemcpyHostToDevice, s));
  FL_TRY_CUDA(cudaMemcpyAsync(m->st_rhs.p, rhs, sizeof(double) * m->N, cudaMemcpyHostToDevice, s));
  FL_TRY_CUDA(cudaMemcpyAsync(m->st_x.p, x, sizeof(double) * m->N, cudaMemcpyHostToDevice, s));
  const uint8_t* ip = nullptr;
  if (inactive) {
    FL_TRY(m->st_ina.reserve(m->N));
    FL_TRY_CUDA(cudaMemcpyAsync(m->st_ina.p, inactive, m->N, cudaMemcpyHostToDevice, s));
    ip = m->st_ina.p;
  }
  FL_TRY(solve(m, o, m->st_val.p, ip, m->st_rhs.p, m->st_x.p, rep, s));
  FL_TRY_CUDA(cudaMemcpyAsync(x, m->st_x.p, sizeof(double) * m->N, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  return FL_OK;
}

extern "C" int fl_dev_csr_mult(fl_mesh m, const double* val, const double* x, double* y, void* stream) {
  FL_CHECK_ARG(m && val && x && y, "null argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : m->stream;
  return csr_mult(m, val, x, y, s);
}

// ------------------------------------------------ projected initial guess --
// The projection method for sequences of right-hand sides (P. F. Fischer,
// "Projection techniques for iterative solution of Ax = b with successive
// right-hand sides", Comput. Methods Appl. Mech. Engrg. 163, 1998): given
// basis vectors v_1..v_k (earlier solutions, a predicted solution), the
// initial guess x0 = V a with (V^T A V) a = V^T b minimises the A-norm of the
// error over span(V) -- the norm CG minimises.  A and b are the ghost-reduced
// system the solve runs on (inactive rows and columns dropped, b lifted), so
// the sums run over active rows only and ghost rows of x0 take the rhs.
namespace fl {

constexpr int kProjMax = 8;
constexpr int kProjVals = kProjMax * (kProjMax + 1) / 2 + kProjMax;

struct ProjArgs {
  int32_t n, k;
  const int32_t* findrm;
  const int32_t* colm;
  const double* val;
  const uint8_t* ghost;
  const double* rhs;
  const double* v[kProjMax];
  double* part;  // per block: the k(k+1)/2 Gram entries (upper triangle, row-major), then the k entries of V^T b
};

// One thread per row: w_l = (A v_l)(row) over active columns, b(row) lifted;
// the row's products v_l w_m (l <= m) and v_l b, summed per block in a fixed
// tree; the blocks' partials are summed in block order by k_proj_reduce.
template <int K>
__global__ void __launch_bounds__(kThreads) k_proj_gram(ProjArgs P) {
  note_launch();
  __shared__ double red[kThreads / 32];
  constexpr int NV = K * (K + 1) / 2 + K;
  double acc[NV];
#pragma unroll
  for (int q = 0; q < NV; ++q) acc[q] = 0.0;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < P.n; row += gridDim.x * blockDim.x) {
    if (P.ghost && P.ghost[row]) continue;
    double w[K], lift = 0.0;
#pragma unroll
    for (int l = 0; l < K; ++l) w[l] = 0.0;
    const int b = __ldg(P.findrm + row), e = __ldg(P.findrm + row + 1);
    for (int q = b; q < e; ++q) {
      const int j = __ldg(P.colm + q);
      const double a = __ldg(P.val + q);
      if (P.ghost && P.ghost[j]) {
        lift += a * P.rhs[j];
        continue;
      }
#pragma unroll
      for (int l = 0; l < K; ++l) w[l] += a * __ldg(P.v[l] + j);
    }
    const double bi = P.rhs[row] - lift;
    double vi[K];
#pragma unroll
    for (int l = 0; l < K; ++l) vi[l] = __ldg(P.v[l] + row);
    int q = 0;
#pragma unroll
    for (int l = 0; l < K; ++l)
#pragma unroll
      for (int m = l; m < K; ++m) acc[q++] += vi[l] * w[m];
#pragma unroll
    for (int l = 0; l < K; ++l) acc[q++] += vi[l] * bi;
  }
#pragma unroll
  for (int q = 0; q < NV; ++q) {
    const double s = block_sum<kThreads>(acc[q], red);
    if (threadIdx.x == 0) P.part[(int64_t)blockIdx.x * NV + q] = s;
  }
}

// The blocks' partials of each value summed in block order (one block).
__global__ void k_proj_reduce(const double* __restrict__ part, int nblocks, int nv, double* __restrict__ out) {
  note_launch();
  __shared__ double red[kThreads / 32];
  for (int q = 0; q < nv; ++q) {
    double s = 0.0;
    for (int b = threadIdx.x; b < nblocks; b += kThreads) s += part[(int64_t)b * nv + q];
    s = block_sum<kThreads>(s, red);
    if (threadIdx.x == 0) out[q] = s;
  }
}

struct ProjCoef {
  double a[kProjMax];
};

__global__ void k_proj_combine(int n, int k, ProjCoef C, ProjArgs P, double* __restrict__ x0) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (P.ghost && P.ghost[i]) {
      x0[i] = P.rhs[i];
      continue;
    }
    double s = 0.0;
    for (int l = 0; l < k; ++l) s += C.a[l] * P.v[l][i];
    x0[i] = s;
  }
}

// (V^T A V) a = V^T b by an LDL^T factorisation that drops a basis vector
// whose pivot is below 1e-13 of its diagonal (it lies in the span of the
// earlier ones): the earlier vectors take precedence.
static void proj_solve(int k, const double* vals, double* a) {
  double G[kProjMax][kProjMax], c[kProjMax], L[kProjMax][kProjMax] = {}, D[kProjMax];
  bool keep[kProjMax];
  int q = 0;
  for (int l = 0; l < k; ++l)
    for (int m = l; m < k; ++m) G[l][m] = G[m][l] = vals[q++];
  for (int l = 0; l < k; ++l) c[l] = vals[q++];
  for (int i = 0; i < k; ++i) {
    double d = G[i][i];
    for (int j = 0; j < i; ++j)
      if (keep[j]) d -= L[i][j] * L[i][j] * D[j];
    keep[i] = G[i][i] > 0.0 && d > 1e-13 * G[i][i];
    D[i] = keep[i] ? d : 0.0;
    L[i][i] = 1.0;
    for (int r = i + 1; r < k; ++r) {
      double s = G[r][i];
      for (int j = 0; j < i; ++j)
        if (keep[j]) s -= L[r][j] * L[i][j] * D[j];
      L[r][i] = keep[i] ? s / D[i] : 0.0;
    }
  }
  double y[kProjMax];
  for (int i = 0; i < k; ++i) {  // L y = c
    double s = c[i];
    for (int j = 0; j < i; ++j) s -= L[i][j] * y[j];
    y[i] = keep[i] ? s : 0.0;
  }
  for (int i = 0; i < k; ++i) y[i] = keep[i] ? y[i] / D[i] : 0.0;
  for (int i = k - 1; i >= 0; --i) {  // L^T a = y
    double s = y[i];
    for (int j = i + 1; j < k; ++j) s -= L[j][i] * a[j];
    a[i] = keep[i] ? s : 0.0;
  }
}

}  // namespace fl

extern "C" int fl_dev_projected_guess(fl_mesh m, const double* val, const uint8_t* inactive, const double* rhs,
                                      int32_t k, const double* const* basis, double* x0, double* coef,
                                      void* stream) {
  using namespace fl;
  FL_CHECK_ARG(m && val && rhs && basis && x0, "null argument");
  FL_CHECK_ARG(k >= 1 && k <= kProjMax, "1 to 8 basis vectors");
  for (int l = 0; l < k; ++l) FL_CHECK_ARG(basis[l], "null basis vector");
  cudaStream_t s = stream ? (cudaStream_t)stream : m->stream;
  KrylovWork* W = work_of(m);
  if (!W) return FL_ERR_NOMEM;
  const unsigned g = grid_for(m->N, kThreads, 4);
  const int nv = k * (k + 1) / 2 + k;
  FL_TRY(W->part.reserve((size_t)g * kProjVals + kProjVals));
  ProjArgs P{};
  P.n = m->N;
  P.k = k;
  P.findrm = m->findrm.p;
  P.colm = m->colm.p;
  P.val = val;
  P.ghost = inactive;
  P.rhs = rhs;
  for (int l = 0; l < k; ++l) P.v[l] = basis[l];
  P.part = W->part.p;
  double* sums = W->part.p + (size_t)g * kProjVals;
  switch (k) {
#define FL_PROJ_CASE(K) \
  case K: k_proj_gram<K><<<g, kThreads, 0, s>>>(P); break;
    FL_PROJ_CASE(1) FL_PROJ_CASE(2) FL_PROJ_CASE(3) FL_PROJ_CASE(4)
    FL_PROJ_CASE(5) FL_PROJ_CASE(6) FL_PROJ_CASE(7) FL_PROJ_CASE(8)
#undef FL_PROJ_CASE
  }
  k_proj_reduce<<<1, kThreads, 0, s>>>(P.part, (int)g, nv, sums);
  FL_TRY_CUDA(cudaGetLastError());
  double vals[kProjVals];
  FL_TRY_CUDA(cudaMemcpyAsync(vals, sums, sizeof(double) * nv, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  ProjCoef C{};
  proj_solve(k, vals, C.a);
  if (coef)
    for (int l = 0; l < k; ++l) coef[l] = C.a[l];
  k_proj_combine<<<g, kThreads, 0, s>>>(m->N, k, C, P, x0);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}
