// fl_mesh.cu -- mesh registration: connectivity upload, node->element lists,
// first-order CSR sparsity, COLOURING_CG1 colouring, colour sets and the P2
// global numbering, all built on the GPU and bit-exact with the reference
// algorithms they replace (cited per kernel).
#include <cstdarg>
#include <cstring>
#include <algorithm>

#include "fl_internal.cuh"
#include "fl_device.cuh"

namespace fl {

static thread_local char g_err[1024] = "";

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int num_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
      sms = 152;
  }
  return sms;
}

// ------------------------------------------------------------------ scan --
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class Tin>
__global__ void k_scan_tile_sums(const Tin* __restrict__ in, int64_t n, int64_t* __restrict__ sums) {
  note_launch();
  __shared__ int64_t red[kScanThreads / 32];
  int64_t base = (int64_t)blockIdx.x * kScanTile;
  int64_t s = 0;
  for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
    int64_t k = base + i;
    if (k < n) s += (int64_t)in[k];
  }
  s = block_sum_i64<kScanThreads>(s, red);
  if (threadIdx.x == 0) sums[blockIdx.x] = s;
}

// Exclusive scan of in[0..n) into out[0..n] (out[n] = total); tile offsets
// come from the scanned tile sums of a previous pass (or are zero).
template <class Tin, class Tout>
__global__ void k_scan_tile(const Tin* __restrict__ in, Tout* __restrict__ out, int64_t n,
                            const int64_t* __restrict__ tile_off) {
  note_launch();
  __shared__ int64_t wt[kScanThreads / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  int64_t v[kScanItems];
  int64_t t = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? (int64_t)in[base + i] : 0;
    t += v[i];
  }
  int64_t incl = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += y;
  }
  if (lane == 31) wt[warp] = incl;
  __syncthreads();
  if (warp == 0) {
    int64_t w = lane < kScanThreads / 32 ? wt[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kScanThreads / 32) wt[lane] = w;
  }
  __syncthreads();
  int64_t ex = incl - t + (warp > 0 ? wt[warp - 1] : 0) + (tile_off ? tile_off[blockIdx.x] : 0);
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i <= n) out[base + i] = (Tout)ex;
    ex += v[i];
  }
}

template <class Tin, class Tout>
static int scan_rec(const Tin* in, Tout* out, int64_t n, cudaStream_t s) {
  int64_t ntiles = (n + 1 + kScanTile - 1) / kScanTile;
  if (ntiles <= 1) {
    k_scan_tile<Tin, Tout><<<1, kScanThreads, 0, s>>>(in, out, n, nullptr);
    FL_TRY_CUDA(cudaGetLastError());
    return FL_OK;
  }
  DevBuf<int64_t> sums, offs;
  FL_TRY(sums.reserve(ntiles));
  FL_TRY(offs.reserve(ntiles + 1));
  k_scan_tile_sums<Tin><<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, n, sums.p);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY((scan_rec<int64_t, int64_t>(sums.p, offs.p, ntiles, s)));
  k_scan_tile<Tin, Tout><<<(unsigned)ntiles, kScanThreads, 0, s>>>(in, out, n, offs.p);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY_CUDA(cudaStreamSynchronize(s));  // temporaries are freed on return
  return FL_OK;
}

int check_err(ErrWord* d_err, cudaStream_t s, const char* what) {
  ErrWord h{0, 0};
  FL_TRY_CUDA(cudaMemcpyAsync(&h, d_err, sizeof(h), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  if (h.code == FL_OK) return FL_OK;
  FL_TRY_CUDA(cudaMemsetAsync(d_err, 0, sizeof(ErrWord), s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  set_error("%s%s (status %d at index %d)", h.code == FL_ERR_TIMEOUT ? "a bounded device wait ran out: " : "",
            what, h.code, h.where);
  return h.code;
}

unsigned long long launches_mesh() { return unit_launches(); }

int exclusive_scan_i32(const int32_t* d_in, int32_t* d_out, int64_t n, cudaStream_t s) {
  DevBuf<int64_t> tmp;
  FL_TRY(tmp.reserve(n + 1));
  FL_TRY((scan_rec<int32_t, int64_t>(d_in, tmp.p, n, s)));
  int64_t total = 0;
  FL_TRY_CUDA(cudaMemcpyAsync(&total, tmp.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  if (total > INT32_MAX) {
    set_error("scan total %lld does not fit in int32", (long long)total);
    return FL_ERR_UNSUPPORTED;
  }
  k_copy_i64_to_i32<<<grid_for(n + 1, 256), 256, 0, s>>>(tmp.p, d_out, n + 1);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  return FL_OK;
}

// ------------------------------------------------------- node -> element --
__global__ void k_check_conn(const int32_t* __restrict__ nd, int64_t n, int32_t nodes,
                             ErrWord* err) {
  note_launch();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    int v = nd[k];
    if (v < 0 || v >= nodes) set_err(err, FL_ERR_ARG, (int32_t)(k));
  }
}

// In place: every entry is read and rewritten by one thread.
__global__ void k_rebase(int32_t* v, int64_t n, int32_t base) {
  note_launch();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    v[k] -= base;
}

__global__ void k_count_incidence(const int32_t* __restrict__ nd, int64_t n,
                                  int32_t* __restrict__ cnt) {
  note_launch();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[nd[k]], 1);
}

// Incidence (element e, local node a) is packed as e*16 + a; sorting the
// packed values sorts a node's list by element id.
__global__ void k_fill_incidence(const int32_t* __restrict__ nd, int64_t n, int loc,
                                 const int32_t* __restrict__ ptr, int32_t* __restrict__ cursor,
                                 int32_t* __restrict__ ne) {
  note_launch();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    int v = nd[k];
    int e = (int)(k / loc), a = (int)(k - (int64_t)e * loc);
    int slot = atomicAdd(&cursor[v], 1);
    ne[ptr[v] + slot] = e * 16 + a;
  }
}

// Each node's incidence list sorted ascending (lists are short: insertion sort).
__global__ void k_sort_lists(const int32_t* __restrict__ ptr, int32_t* __restrict__ ne, int32_t n) {
  note_launch();
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    int b = ptr[v], e = ptr[v + 1];
    for (int i = b + 1; i < e; ++i) {
      int x = ne[i];
      int j = i - 1;
      while (j >= b && ne[j] > x) {
        ne[j + 1] = ne[j];
        --j;
      }
      ne[j + 1] = x;
    }
  }
}

// node -> incidence lists of a connectivity (0-based, validated).
static int build_incidence(const int32_t* d_nd, int32_t E, int loc, int32_t nodes,
                           DevBuf<int32_t>& ptr, DevBuf<int32_t>& ne, cudaStream_t s) {
  const int64_t n = (int64_t)E * loc;
  DevBuf<int32_t> cnt;
  FL_TRY(cnt.reserve(nodes + 1));
  FL_TRY(ptr.reserve(nodes + 1));
  FL_TRY(ne.reserve(n));
  FL_TRY_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (nodes + 1), s));
  k_count_incidence<<<grid_for(n, 256), 256, 0, s>>>(d_nd, n, cnt.p);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY(exclusive_scan_i32(cnt.p, ptr.p, nodes, s));
  FL_TRY_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (nodes + 1), s));
  k_fill_incidence<<<grid_for(n, 256), 256, 0, s>>>(d_nd, n, loc, ptr.p, cnt.p, ne.p);
  FL_TRY_CUDA(cudaGetLastError());
  k_sort_lists<<<grid_for(nodes, 128), 128, 0, s>>>(ptr.p, ne.p, nodes);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  return FL_OK;
}

// -------------------------------------------------------------- sparsity --
// make_sparsity_lists / lists2csr_sparsity (Sparsity_Patterns.F90:299-430):
// row i holds every node sharing an element with i, ascending, no repeats.
// One warp per row: candidates from the row's incidences are staged in shared
// memory, bitonic-sorted, and de-duplicated.  Pass 0 counts, pass 1 writes
// colm and centrm.
constexpr int kRowWarps = 4;
constexpr int kRowCap = 2048;

__global__ void __launch_bounds__(kRowWarps * 32)
k_sparsity_rows(const int32_t* __restrict__ ne_ptr, const int32_t* __restrict__ ne,
                const int32_t* __restrict__ nd, int loc, int32_t nrows, int pass,
                int32_t* __restrict__ counts, const int32_t* __restrict__ findrm,
                int32_t* __restrict__ colm, int32_t* __restrict__ centrm, ErrWord* err) {
  note_launch();
  __shared__ int32_t buf[kRowWarps][kRowCap];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t* s = buf[w];
  for (int row = blockIdx.x * kRowWarps + w; row < nrows; row += gridDim.x * kRowWarps) {
    const int b = ne_ptr[row], deg = ne_ptr[row + 1] - b;
    const int ncand = deg * loc;
    if (ncand > kRowCap) {
      if (lane == 0) set_err(err, FL_ERR_UNSUPPORTED, row);
      continue;
    }
    int P = 32;
    while (P < ncand) P <<= 1;
    for (int idx = lane; idx < P; idx += 32) {
      int v = INT32_MAX;
      if (idx < ncand) {
        int inc = ne[b + idx / loc];
        v = nd[(int64_t)(inc >> 4) * loc + (idx % loc)];
      }
      s[idx] = v;
    }
    __syncwarp();
    for (int k = 2; k <= P; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int idx = lane; idx < P; idx += 32) {
          int ixj = idx ^ j;
          if (ixj > idx) {
            int a = s[idx], c = s[ixj];
            bool up = (idx & k) == 0;
            if ((a > c) == up) {
              s[idx] = c;
              s[ixj] = a;
            }
          }
        }
        __syncwarp();
      }
    int running = 0;
    const int out0 = pass ? findrm[row] : 0;
    int diag = -1;
    for (int base = 0; base < P; base += 32) {
      int idx = base + lane;
      int v = s[idx];
      bool keep = v != INT32_MAX && (idx == 0 || v != s[idx - 1]);
      unsigned m = __ballot_sync(0xffffffffu, keep);
      if (pass && keep) {
        int pos = out0 + running + __popc(m & ((1u << lane) - 1u));
        colm[pos] = v;
        if (v == row) diag = pos;
      }
      running += __popc(m);
    }
    if (pass) {
      unsigned dm = __ballot_sync(0xffffffffu, diag >= 0);
      int d = dm ? __shfl_sync(0xffffffffu, diag, __ffs(dm) - 1) : -1;
      if (lane == 0) centrm[row] = d;
    } else if (lane == 0) {
      counts[row] = running;
    }
    __syncwarp();
  }
}

static int build_sparsity(const int32_t* d_nd, int loc, int32_t nrows, const DevBuf<int32_t>& ne_ptr,
                          const DevBuf<int32_t>& ne, DevBuf<int32_t>& findrm, DevBuf<int32_t>& colm,
                          DevBuf<int32_t>& centrm, int64_t* nnz, ErrWord* d_err, cudaStream_t s) {
  DevBuf<int32_t> cnt;
  FL_TRY(cnt.reserve(nrows + 1));
  FL_TRY(findrm.reserve(nrows + 1));
  FL_TRY(centrm.reserve(nrows));
  unsigned g = grid_for((int64_t)nrows, kRowWarps, 16);
  k_sparsity_rows<<<g, kRowWarps * 32, 0, s>>>(ne_ptr.p, ne.p, d_nd, loc, nrows, 0, cnt.p, nullptr,
                                               nullptr, nullptr, d_err);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY(check_err(d_err, s, "sparsity row"));
  FL_TRY(exclusive_scan_i32(cnt.p, findrm.p, nrows, s));
  int32_t total = 0;
  FL_TRY_CUDA(cudaMemcpyAsync(&total, findrm.p + nrows, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  FL_TRY(colm.reserve(total));
  k_sparsity_rows<<<g, kRowWarps * 32, 0, s>>>(ne_ptr.p, ne.p, d_nd, loc, nrows, 1, nullptr,
                                               findrm.p, colm.p, centrm.p, d_err);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY(check_err(d_err, s, "sparsity fill"));
  *nnz = total;
  return FL_OK;
}

// ------------------------------------------------------------- colouring --
// COLOURING_CG1 (Colouring.F90:85-199): element e takes the lowest colour >= 1
// not used by any lower-numbered element sharing a vertex with it.  This is
// the unique fixed point of c(e) = mex{c(f) : f < e, f ~ e}; it is computed as
// a dataflow over the element order: warps take elements in ascending order
// from a ticket counter, wait (bounded) until every lower neighbour has its
// colour, and publish their own.  Every wait is on a lower ticket already held
// by a running warp, so the lowest unfinished element can always proceed.
constexpr int kMaxColourWords = 8;  // up to 256 colours

__global__ void k_colour_dataflow(const int32_t* __restrict__ vne_ptr, const int32_t* __restrict__ vne,
                                  const int32_t* __restrict__ xnd, int32_t E,
                                  int32_t* __restrict__ colour, int32_t* __restrict__ ticket,
                                  ErrWord* err, long long wait_cycles, int32_t withhold) {
  note_launch();
  const int lane = threadIdx.x & 31;
  while (true) {
    int e = 0;
    if (lane == 0) e = atomicAdd(ticket, 1);
    e = __shfl_sync(0xffffffffu, e, 0);
    if (e >= E) return;
    uint32_t mask[kMaxColourWords];
#pragma unroll
    for (int k = 0; k < kMaxColourWords; ++k) mask[k] = 0u;
    bool bad = false;
    for (int j = 0; j < 4; ++j) {
      const int v = xnd[(int64_t)e * 4 + j];
      const int b = vne_ptr[v], end = vne_ptr[v + 1];
      for (int idx = b + lane; idx < end; idx += 32) {
        const int f = vne[idx] >> 4;
        if (f >= e) continue;
        int c = ld_relaxed(&colour[f]);
        if (c == 0) {
          long long t0 = clock64();
          while ((c = ld_relaxed(&colour[f])) == 0) {
            if (ld_relaxed(&err->code) != FL_OK) {
              bad = true;
              break;
            }
            if (clock64() - t0 > wait_cycles) {
              set_err(err, FL_ERR_TIMEOUT, e);
              bad = true;
              break;
            }
            __nanosleep(64);
          }
        }
        if (bad) break;
        if (c > 32 * kMaxColourWords) {
          bad = true;
          set_err(err, FL_ERR_COLOURS, e);
          break;
        }
        mask[(c - 1) >> 5] |= 1u << ((c - 1) & 31);
      }
      if (bad) break;
    }
    if (__any_sync(0xffffffffu, bad)) return;  // status already recorded
    int mine = 0;
#pragma unroll
    for (int k = 0; k < kMaxColourWords; ++k) {
      uint32_t m = __reduce_or_sync(0xffffffffu, mask[k]);
      if (!mine && m != 0xffffffffu) mine = 32 * k + __ffs(~m);
    }
    if (lane == 0 && e != withhold) {  // a withheld element (failure-injection test) never publishes
      if (mine == 0) {
        set_err(err, FL_ERR_COLOURS, e);
        st_relaxed(&colour[e], 1 << 30);  // unblock waiters; status reports the failure
      } else {
        st_relaxed(&colour[e], mine);
      }
    }
  }
}

__global__ void k_colour_hist(const int32_t* __restrict__ colour, int32_t E, int32_t* __restrict__ hist,
                              int32_t* __restrict__ maxc) {
  note_launch();
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
    int c = colour[e];
    atomicAdd(&hist[c], 1);
    atomicMax(maxc, c);
  }
}

__global__ void k_flag_colour(const int32_t* __restrict__ colour, int32_t E, int c,
                              int32_t* __restrict__ flag) {
  note_launch();
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x)
    flag[e] = colour[e] == c;
}

__global__ void k_scatter_colour(const int32_t* __restrict__ colour, int32_t E, int c,
                                 const int32_t* __restrict__ pos, int32_t base,
                                 int32_t* __restrict__ out) {
  note_launch();
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x)
    if (colour[e] == c) out[base + pos[e]] = e;
}

// Each node's incidences reordered by the colour of their element.  A node
// meets at most one element of each colour, so the order is total; it is the
// order in which the reference's coloured loop (Advection_Diffusion_CG.F90:582-598)
// adds the elements' contributions to that node's row.
__global__ void k_sort_by_colour(const int32_t* __restrict__ ptr, const int32_t* __restrict__ ne,
                                 const int32_t* __restrict__ colour, int32_t* __restrict__ out, int32_t n) {
  note_launch();
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
    const int b = ptr[v], e = ptr[v + 1];
    for (int i = b; i < e; ++i) out[i] = ne[i];
    for (int i = b + 1; i < e; ++i) {
      const int x = out[i];
      const int cx = colour[x >> 4];
      int j = i - 1;
      while (j >= b && colour[out[j] >> 4] > cx) {
        out[j + 1] = out[j];
        --j;
      }
      out[j + 1] = x;
    }
  }
}

// For every incidence (row i, element e) of ne_col, the positions of e's nodes
// inside row i (offsets from findrm[i]), one byte each -- the bisection of
// csr_sparsity_pos (Sparse_Tools.F90:2411) done once per mesh instead of once
// per entry per assembly.  255 marks a position that does not fit a byte.
__global__ void k_incidence_positions(const int32_t* __restrict__ ne_ptr, const int32_t* __restrict__ ne_col,
                                      const int32_t* __restrict__ nd, int loc, const int32_t* __restrict__ findrm,
                                      const int32_t* __restrict__ colm, int32_t n, uint32_t* __restrict__ pos,
                                      ErrWord* err) {
  note_launch();
  const int pw = (loc + 3) / 4;
  for (int row = blockIdx.x * blockDim.x + threadIdx.x; row < n; row += gridDim.x * blockDim.x) {
    const int b0 = findrm[row], b1 = findrm[row + 1];
    for (int q = ne_ptr[row]; q < ne_ptr[row + 1]; ++q) {
      const int e = ne_col[q] >> 4;
      uint32_t words[3] = {0u, 0u, 0u};
      for (int b = 0; b < loc; ++b) {
        const int j = nd[(int64_t)e * loc + b];
        const int p = csr_find(colm, b0, b1, j);
        if (p < 0) set_err(err, FL_ERR_OUTSIDE_PATTERN, row);
        if (p - b0 > 254) set_err(err, FL_ERR_UNSUPPORTED, row);  // rows longer than 255 entries
        const uint32_t off = p < 0 ? 255u : (uint32_t)min(p - b0, 255);
        words[b >> 2] |= off << (8 * (b & 3));
      }
      for (int w = 0; w < pw; ++w) pos[(int64_t)q * pw + w] = words[w];
    }
  }
}

WaitTest& wait_test() {
  static WaitTest w;
  return w;
}

static int build_colouring(fl_mesh_t* m, cudaStream_t s) {
  const int32_t E = m->E;
  FL_TRY(m->vne_ptr.reserve(m->Nx + 1));
  FL_TRY(build_incidence(m->xndglno.p, E, 4, m->Nx, m->vne_ptr, m->vne, s));
  FL_TRY(m->colour.reserve(E));
  FL_TRY_CUDA(cudaMemsetAsync(m->colour.p, 0, sizeof(int32_t) * E, s));
  DevBuf<int32_t> ticket;
  FL_TRY(ticket.reserve(2));
  FL_TRY_CUDA(cudaMemsetAsync(ticket.p, 0, sizeof(int32_t) * 2, s));
  int dev = 0, clk_khz = 2000000;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&clk_khz, cudaDevAttrClockRate, dev);
  const WaitTest& wt = wait_test();
  const long long wait_cycles = wt.wait_ms > 0.0 ? (long long)(clk_khz * wt.wait_ms)
                                                 : (long long)clk_khz * 1000LL * 2;  // ~2 s per wait
  k_colour_dataflow<<<num_sms() * 8, 256, 0, s>>>(m->vne_ptr.p, m->vne.p, m->xndglno.p, E,
                                                   m->colour.p, ticket.p, m->err.p, wait_cycles, wt.withhold);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY(check_err(m->err.p, s, "colouring"));
  // colour sets: histogram, offsets, stable per-colour compaction
  DevBuf<int32_t> hist;
  FL_TRY(hist.reserve(32 * kMaxColourWords + 2));
  FL_TRY_CUDA(cudaMemsetAsync(hist.p, 0, sizeof(int32_t) * (32 * kMaxColourWords + 2), s));
  k_colour_hist<<<grid_for(E, 256), 256, 0, s>>>(m->colour.p, E, hist.p,
                                                  hist.p + 32 * kMaxColourWords + 1);
  FL_TRY_CUDA(cudaGetLastError());
  std::vector<int32_t> h(32 * kMaxColourWords + 2);
  FL_TRY_CUDA(cudaMemcpyAsync(h.data(), hist.p, sizeof(int32_t) * h.size(), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  const int ncol = h.back();
  m->ncolours = ncol;
  m->colour_ptr.assign(ncol + 1, 0);
  for (int c = 1; c <= ncol; ++c) m->colour_ptr[c] = m->colour_ptr[c - 1] + h[c];
  FL_TRY(m->colour_elems.reserve(E));
  DevBuf<int32_t> flag, pos;
  FL_TRY(flag.reserve(E + 1));
  FL_TRY(pos.reserve(E + 1));
  for (int c = 1; c <= ncol; ++c) {
    k_flag_colour<<<grid_for(E, 256), 256, 0, s>>>(m->colour.p, E, c, flag.p);
    FL_TRY_CUDA(cudaGetLastError());
    FL_TRY(exclusive_scan_i32(flag.p, pos.p, E, s));
    k_scatter_colour<<<grid_for(E, 256), 256, 0, s>>>(m->colour.p, E, c, pos.p,
                                                       m->colour_ptr[c - 1], m->colour_elems.p);
    FL_TRY_CUDA(cudaGetLastError());
  }
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  return FL_OK;
}

// ---------------------------------------------------------- P2 numbering --
// make_global_numbering, serial (Global_Numbering.F90:453-634):
//  * vertex v gets the rank of its first touch (element-major position) among
//    all first touches -- the first-touch renumbering of :460-493;
//  * edge (i, j), i < j in old numbering, gets N1 + (number of edges (i', j')
//    with i' < i) + (rank of j among row i's neighbours greater than i): the
//    (old node ascending, NNList ascending) order of :497-634, read off the
//    sorted P1 CSR pattern (upper triangle counts).
__global__ void k_first_touch(const int32_t* __restrict__ nd, int64_t n, int32_t* __restrict__ first) {
  note_launch();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    atomicMin(&first[nd[k]], (int32_t)k);
}

__global__ void k_mark_first(const int32_t* __restrict__ first, int32_t nv, int32_t* __restrict__ mark,
                             ErrWord* err) {
  note_launch();
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
    int f = first[v];
    if (f == INT32_MAX) set_err(err, FL_ERR_ARG, v);  // vertex used by no element
    else mark[f] = 1;
  }
}

__global__ void k_upper_counts(const int32_t* __restrict__ findrm, const int32_t* __restrict__ centrm,
                               int32_t n, int32_t* __restrict__ up) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    up[i] = findrm[i + 1] - centrm[i] - 1;
}

__global__ void k_p2_numbering(const int32_t* __restrict__ nd1, int32_t E, const int32_t* __restrict__ first,
                               const int32_t* __restrict__ rankpos, const int32_t* __restrict__ findrm,
                               const int32_t* __restrict__ colm, const int32_t* __restrict__ centrm,
                               const int32_t* __restrict__ uoff, int32_t nv, int32_t out_base,
                               int32_t* __restrict__ nd2) {
  note_launch();
  // number_tets_lagrange positions (Element_Numbering.F90:389-472)
  const int vpos[4] = {0, 2, 5, 9};
  const int epos[4][4] = {{-1, 1, 3, 6}, {1, -1, 4, 7}, {3, 4, -1, 8}, {6, 7, 8, -1}};
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
    int v[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) v[a] = nd1[(int64_t)e * 4 + a];
#pragma unroll
    for (int a = 0; a < 4; ++a) nd2[(int64_t)e * 10 + vpos[a]] = rankpos[first[v[a]]] + out_base;
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = a + 1; b < 4; ++b) {
        int i = min(v[a], v[b]), j = max(v[a], v[b]);
        int p = csr_find(colm, findrm[i], findrm[i + 1], j);
        nd2[(int64_t)e * 10 + epos[a][b]] = nv + uoff[i] + (p - centrm[i] - 1) + out_base;
      }
  }
}

}  // namespace fl

using namespace fl;

extern "C" const char* fl_last_error(void) { return g_err; }

__global__ void k_max_row(const int32_t* __restrict__ findrm, int32_t n, int32_t* __restrict__ out) {
  note_launch();
  int m = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    m = max(m, findrm[i + 1] - findrm[i]);
  atomicMax(out, m);
}

static int upload_conn(const int32_t* host, int64_t n, int32_t base, int32_t nodes, DevBuf<int32_t>& dst,
                       ErrWord* d_err, cudaStream_t s) {
  FL_TRY(dst.reserve(n));
  FL_TRY_CUDA(cudaMemcpyAsync(dst.p, host, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s));
  if (base != 0) {
    k_rebase<<<grid_for(n, 256), 256, 0, s>>>(dst.p, n, base);
    FL_TRY_CUDA(cudaGetLastError());
  }
  k_check_conn<<<grid_for(n, 256), 256, 0, s>>>(dst.p, n, nodes, d_err);
  FL_TRY_CUDA(cudaGetLastError());
  return check_err(d_err, s, "connectivity out of range");
}

// Pattern check of a caller's CSR: rows strictly ascending and in range,
// the diagonal's position (-1 when the row has none).
__global__ void k_pattern_check(const int32_t* __restrict__ findrm, const int32_t* __restrict__ colm, int32_t n,
                                int32_t* __restrict__ centrm, ErrWord* err) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int b = findrm[i], e = findrm[i + 1];
    int d = -1;
    if (e < b) set_err(err, FL_ERR_ARG, i);
    for (int k = b; k < e; ++k) {
      const int c = colm[k];
      if (c < 0 || c >= n || (k > b && colm[k - 1] >= c)) set_err(err, FL_ERR_ARG, i);
      if (c == i) d = k;
    }
    centrm[i] = d;
  }
}

// A handle that carries only a square CSR pattern (no elements): enough for
// fl_gpu/dev_petsc_solve and fl_dev_csr_mult on a matrix read from a file.
extern "C" int fl_gpu_pattern_register(int32_t n, const int32_t* findrm, const int32_t* colm, int32_t index_base,
                                       fl_mesh* out) {
  FL_CHECK_ARG(out && findrm && colm, "null argument");
  FL_CHECK_ARG(n > 0, "row count");
  FL_CHECK_ARG(index_base == 0 || index_base == 1, "index_base");
  const int64_t nnz = (int64_t)findrm[n] - findrm[0];
  FL_CHECK_ARG(findrm[0] == index_base && nnz > 0 && nnz < ((int64_t)1 << 31), "row pointers");
  fl_mesh_t* m = new fl_mesh_t();
  int st = FL_OK;
  do {
    cudaGetDevice(&m->device);
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) {
      set_error("cudaStreamCreate failed");
      st = FL_ERR_CUDA;
      break;
    }
    cudaStream_t s = m->stream;
    m->N = n;
    m->nnz = nnz;
    std::vector<int32_t> f(n + 1), c((size_t)nnz);
    for (int i = 0; i <= n; ++i) f[i] = findrm[i] - index_base;
    for (int64_t k = 0; k < nnz; ++k) c[k] = colm[k] - index_base;
    int32_t mr = 0;
    for (int i = 0; i < n; ++i) mr = std::max(mr, f[i + 1] - f[i]);
    m->max_row = mr;
    if ((st = m->err.reserve(1)) || (st = m->findrm.reserve(n + 1)) || (st = m->colm.reserve(nnz)) ||
        (st = m->centrm.reserve(n)))
      break;
    if (cudaMemsetAsync(m->err.p, 0, sizeof(ErrWord), s) != cudaSuccess ||
        cudaMemcpyAsync(m->findrm.p, f.data(), sizeof(int32_t) * (n + 1), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(m->colm.p, c.data(), sizeof(int32_t) * nnz, cudaMemcpyHostToDevice, s) != cudaSuccess) {
      set_error("pattern upload failed");
      st = FL_ERR_CUDA;
      break;
    }
    k_pattern_check<<<grid_for(n, 256), 256, 0, s>>>(m->findrm.p, m->colm.p, n, m->centrm.p, m->err.p);
    if ((st = check_err(m->err.p, s, "CSR rows must hold ascending column indices in range")) != FL_OK) break;
  } while (0);
  if (st != FL_OK) {
    fl_gpu_mesh_destroy(m);
    return st;
  }
  *out = m;
  return FL_OK;
}

extern "C" int fl_gpu_mesh_register(const fl_mesh_desc* d, fl_mesh* out) {
  FL_CHECK_ARG(d && out, "null descriptor/handle");
  FL_CHECK_ARG(d->loc == 4 || d->loc == 10, "loc must be 4 (P1) or 10 (P2)");
  FL_CHECK_ARG(d->elements > 0 && d->elements < (1 << 27), "element count out of range");
  FL_CHECK_ARG(d->nodes > 0 && d->x_nodes > 0, "node counts");
  FL_CHECK_ARG(d->ndglno && d->coords, "ndglno/coords");
  FL_CHECK_ARG(d->index_base == 0 || d->index_base == 1, "index_base");
  FL_CHECK_ARG(d->loc == 4 || d->x_ndglno, "P2 meshes need the coordinate connectivity");
  fl_mesh_t* m = new fl_mesh_t();
  int st = FL_OK;
  do {
    cudaGetDevice(&m->device);
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) {
      set_error("cudaStreamCreate failed");
      st = FL_ERR_CUDA;
      break;
    }
    cudaStream_t s = m->stream;
    m->N = d->nodes;
    m->E = d->elements;
    m->loc = d->loc;
    m->Nx = d->x_nodes;
    if ((st = m->err.reserve(1)) != FL_OK) break;
    if (cudaMemsetAsync(m->err.p, 0, sizeof(ErrWord), s) != cudaSuccess) { st = FL_ERR_CUDA; break; }
    const int32_t* xnd = d->x_ndglno ? d->x_ndglno : d->ndglno;
    if ((st = upload_conn(d->ndglno, (int64_t)m->E * m->loc, d->index_base, m->N, m->ndglno, m->err.p, s)) != FL_OK) break;
    if ((st = upload_conn(xnd, (int64_t)m->E * 4, d->index_base, m->Nx, m->xndglno, m->err.p, s)) != FL_OK) break;
    if ((st = m->coords.reserve((size_t)3 * m->Nx)) != FL_OK) break;
    if (cudaMemcpyAsync(m->coords.p, d->coords, sizeof(double) * 3 * m->Nx, cudaMemcpyHostToDevice, s) != cudaSuccess) {
      set_error("coords upload failed");
      st = FL_ERR_CUDA;
      break;
    }
    if ((st = build_incidence(m->ndglno.p, m->E, m->loc, m->N, m->ne_ptr, m->ne, s)) != FL_OK) break;
    if ((st = build_sparsity(m->ndglno.p, m->loc, m->N, m->ne_ptr, m->ne, m->findrm, m->colm, m->centrm,
                             &m->nnz, m->err.p, s)) != FL_OK) break;
    {
      DevBuf<int32_t> mr;
      if ((st = mr.reserve(1)) != FL_OK) break;
      cudaMemsetAsync(mr.p, 0, sizeof(int32_t), s);
      k_max_row<<<grid_for(m->N, 256), 256, 0, s>>>(m->findrm.p, m->N, mr.p);
      if (cudaMemcpyAsync(&m->max_row, mr.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
          cudaStreamSynchronize(s) != cudaSuccess) {
        set_error("row length reduction failed");
        st = FL_ERR_CUDA;
        break;
      }
    }
    if ((st = build_colouring(m, s)) != FL_OK) break;
    if ((st = m->ne_col.reserve((size_t)m->E * m->loc)) != FL_OK) break;
    k_sort_by_colour<<<grid_for(m->N, 128), 128, 0, s>>>(m->ne_ptr.p, m->ne.p, m->colour.p, m->ne_col.p, m->N);
    if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetLastError() != cudaSuccess) {
      set_error("colour ordering of incidences failed");
      st = FL_ERR_CUDA;
      break;
    }
    if ((st = m->ne_pos.reserve((size_t)m->E * m->loc * ((m->loc + 3) / 4))) != FL_OK) break;
    k_incidence_positions<<<grid_for(m->N, 128), 128, 0, s>>>(m->ne_ptr.p, m->ne_col.p, m->ndglno.p, m->loc,
                                                              m->findrm.p, m->colm.p, m->N, m->ne_pos.p, m->err.p);
    if ((st = check_err(m->err.p, s, "incidence positions")) != FL_OK) break;
  } while (0);
  if (st != FL_OK) {
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return st;
  }
  *out = m;
  return FL_OK;
}

extern "C" int fl_gpu_mesh_destroy(fl_mesh m) {
  if (!m) return FL_OK;
  cudaStreamSynchronize(m->stream);
  release_krylov_work(m);
  if (m->ev0) cudaEventDestroy(m->ev0);
  if (m->ev1) cudaEventDestroy(m->ev1);
  for (cudaStream_t q : m->ck_streams)
    if (q) {
      cudaStreamSynchronize(q);
      cudaStreamDestroy(q);
    }
  for (cudaEvent_t e : m->ck_ev) cudaEventDestroy(e);
  cudaStreamDestroy(m->stream);
  delete m;
  return FL_OK;
}

extern "C" int64_t fl_kernel_launch_count(void) {
  return (int64_t)(launches_mesh() + launches_assemble() + launches_krylov() + launches_gnn() +
                   launches_amg() + launches_projection());
}

extern "C" int fl_gpu_mesh_info(fl_mesh m, int64_t* nnz, int32_t* ncolours) {
  FL_CHECK_ARG(m, "null mesh");
  if (nnz) *nnz = m->nnz;
  if (ncolours) *ncolours = m->ncolours;
  return FL_OK;
}

__global__ void k_offset_copy(const int32_t* __restrict__ in, int32_t* __restrict__ out, int64_t n,
                              int32_t add, int32_t missing_in, int32_t missing_out) {
  note_launch();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x) {
    int v = in[k];
    out[k] = (v == missing_in) ? missing_out : v + add;
  }
}

static int copy_out(const int32_t* d, int64_t n, int32_t add, int32_t* host, cudaStream_t s,
                    bool centrm = false) {
  DevBuf<int32_t> tmp;
  FL_TRY(tmp.reserve(n));
  // a missing diagonal is -1 on the device; 0 in base 1 (lists2csr_sparsity), -1 in base 0
  k_offset_copy<<<grid_for(n, 256), 256, 0, s>>>(d, tmp.p, n, add, centrm ? -1 : INT32_MIN,
                                                  centrm ? (add ? 0 : -1) : INT32_MIN);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY_CUDA(cudaMemcpyAsync(host, tmp.p, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  return FL_OK;
}

extern "C" int fl_gpu_sparsity_copy(fl_mesh m, int32_t* findrm, int32_t* colm, int32_t* centrm,
                                    int32_t base) {
  FL_CHECK_ARG(m, "null mesh");
  FL_CHECK_ARG(base == 0 || base == 1, "index_base");
  if (findrm) FL_TRY(copy_out(m->findrm.p, m->N + 1, base, findrm, m->stream));
  if (colm) FL_TRY(copy_out(m->colm.p, m->nnz, base, colm, m->stream));
  if (centrm) FL_TRY(copy_out(m->centrm.p, m->N, base, centrm, m->stream, true));
  return FL_OK;
}

extern "C" int fl_gpu_colouring_copy(fl_mesh m, int32_t* colour, int32_t* colour_ptr,
                                     int32_t* colour_elems, int32_t base) {
  FL_CHECK_ARG(m, "null mesh");
  FL_CHECK_ARG(base == 0 || base == 1, "index_base");
  if (colour) {
    FL_TRY_CUDA(cudaMemcpyAsync(colour, m->colour.p, sizeof(int32_t) * m->E, cudaMemcpyDeviceToHost, m->stream));
    FL_TRY_CUDA(cudaStreamSynchronize(m->stream));
  }
  if (colour_ptr)
    for (int c = 0; c <= m->ncolours; ++c) colour_ptr[c] = m->colour_ptr[c] + base;
  if (colour_elems) FL_TRY(copy_out(m->colour_elems.p, m->E, base, colour_elems, m->stream));
  return FL_OK;
}

extern "C" int fl_gpu_make_global_numbering_p2(int32_t nv, int32_t E, const int32_t* nd1_host,
                                               int32_t base, int32_t* nd2_host, int32_t* n2) {
  FL_CHECK_ARG(nd1_host && nd2_host && n2, "null pointer");
  FL_CHECK_ARG(nv > 0 && E > 0 && E < (1 << 27), "sizes");
  FL_CHECK_ARG(base == 0 || base == 1, "index_base");
  cudaStream_t s;
  FL_TRY_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  struct StreamGuard {
    cudaStream_t s;
    ~StreamGuard() { cudaStreamSynchronize(s); cudaStreamDestroy(s); }
  } guard{s};
  DevBuf<ErrWord> err;
  FL_TRY(err.reserve(1));
  FL_TRY_CUDA(cudaMemsetAsync(err.p, 0, sizeof(ErrWord), s));
  DevBuf<int32_t> nd1, ptr, ne, findrm, colm, centrm, first, mark, rankpos, up, uoff, nd2;
  const int64_t n = (int64_t)E * 4;
  FL_TRY(upload_conn(nd1_host, n, base, nv, nd1, err.p, s));
  FL_TRY(build_incidence(nd1.p, E, 4, nv, ptr, ne, s));
  int64_t nnz = 0;
  FL_TRY(build_sparsity(nd1.p, 4, nv, ptr, ne, findrm, colm, centrm, &nnz, err.p, s));
  FL_TRY(first.reserve(nv));
  FL_TRY(mark.reserve(n + 1));
  FL_TRY(rankpos.reserve(n + 1));
  k_fill_i32<<<grid_for(nv, 256), 256, 0, s>>>(first.p, nv, INT32_MAX);
  FL_TRY_CUDA(cudaMemsetAsync(mark.p, 0, sizeof(int32_t) * (n + 1), s));
  k_first_touch<<<grid_for(n, 256), 256, 0, s>>>(nd1.p, n, first.p);
  k_mark_first<<<grid_for(nv, 256), 256, 0, s>>>(first.p, nv, mark.p, err.p);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY(check_err(err.p, s, "unused vertex in P1 connectivity"));
  FL_TRY(exclusive_scan_i32(mark.p, rankpos.p, n, s));
  FL_TRY(up.reserve(nv + 1));
  FL_TRY(uoff.reserve(nv + 1));
  k_upper_counts<<<grid_for(nv, 256), 256, 0, s>>>(findrm.p, centrm.p, nv, up.p);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY(exclusive_scan_i32(up.p, uoff.p, nv, s));
  int32_t nedges = 0;
  FL_TRY_CUDA(cudaMemcpyAsync(&nedges, uoff.p + nv, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FL_TRY(nd2.reserve((size_t)E * 10));
  k_p2_numbering<<<grid_for(E, 256), 256, 0, s>>>(nd1.p, E, first.p, rankpos.p, findrm.p, colm.p, centrm.p,
                                                   uoff.p, nv, base, nd2.p);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY_CUDA(cudaMemcpyAsync(nd2_host, nd2.p, sizeof(int32_t) * (size_t)E * 10, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  *n2 = nv + nedges;
  return FL_OK;
}

extern "C" int fl_set_wait_test(int32_t withhold, double wait_ms) {
  using namespace fl;
  FL_CHECK_ARG(withhold >= -1, "withhold is a flag index, or -1 to switch the hook off");
  FL_CHECK_ARG(wait_ms >= 0.0 && wait_ms <= 60000.0, "wait_ms in [0, 60000]");
  FL_CHECK_ARG(withhold == -1 || wait_ms > 0.0, "a withheld flag needs a wait limit (wait_ms > 0)");
  wait_test().withhold = withhold;
  wait_test().wait_ms = wait_ms;
  return FL_OK;
}

// make_sparsity(pressure mesh, velocity mesh) (femtools/Sparsity_Patterns.F90
// :47-85) for P1 pressure on the vertices and P2 velocity of one P2 mesh
// handle: row v (a vertex of the coordinate mesh) holds the P2 nodes of the
// elements containing v, ascending -- the first-order builder run over the
// vertex -> element incidences with the P2 connectivity as candidates.
extern "C" int fl_gpu_rect_register(fl_mesh m, fl_mesh* out) {
  using namespace fl;
  FL_CHECK_ARG(m && out, "null argument");
  FL_CHECK_ARG(m->loc == 10 && m->E > 0 && m->vne_ptr.p, "a registered P2 mesh handle");
  fl_mesh_t* h = new fl_mesh_t();
  int st = FL_OK;
  do {
    cudaGetDevice(&h->device);
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
      set_error("cudaStreamCreate failed");
      st = FL_ERR_CUDA;
      break;
    }
    cudaStream_t s = h->stream;
    h->N = m->Nx;
    h->so_parent = m;
    if ((st = h->err.reserve(1)) != FL_OK) break;
    if (cudaMemsetAsync(h->err.p, 0, sizeof(ErrWord), s) != cudaSuccess) {
      st = FL_ERR_CUDA;
      break;
    }
    // the velocity mesh's incidences are complete on its own stream
    if (cudaStreamSynchronize(m->stream) != cudaSuccess) {
      st = FL_ERR_CUDA;
      break;
    }
    if ((st = build_sparsity(m->ndglno.p, 10, m->Nx, m->vne_ptr, m->vne, h->findrm, h->colm, h->centrm, &h->nnz,
                             h->err.p, s)) != FL_OK)
      break;
    DevBuf<int32_t> mr;
    if ((st = mr.reserve(1)) != FL_OK) break;
    cudaMemsetAsync(mr.p, 0, sizeof(int32_t), s);
    k_max_row<<<grid_for(h->N, 256), 256, 0, s>>>(h->findrm.p, h->N, mr.p);
    if (cudaMemcpyAsync(&h->max_row, mr.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      set_error("rectangular pattern: row length read failed");
      st = FL_ERR_CUDA;
      break;
    }
  } while (0);
  if (st != FL_OK) {
    fl_gpu_mesh_destroy(h);
    return st;
  }
  *out = h;
  return FL_OK;
}
