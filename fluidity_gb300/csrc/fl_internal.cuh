// fl_internal.cuh -- internal types and helpers of the GB300 CG hot-path
// library.  Not part of the public C-ABI (see include/fluidity_gb300.h).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/fluidity_gb300.h"

namespace fl {

// Last error message of the calling host thread (fl_last_error()).
void set_error(const char* fmt, ...);

#define FL_TRY_CUDA(call)                                                          \
  do {                                                                             \
    cudaError_t _e = (call);                                                       \
    if (_e != cudaSuccess) {                                                       \
      ::fl::set_error("%s:%d: %s: %s", __FILE__, __LINE__, #call,                   \
                      cudaGetErrorString(_e));                                     \
      return FL_ERR_CUDA;                                                          \
    }                                                                              \
  } while (0)

#define FL_TRY(call)                                                               \
  do {                                                                             \
    int _s = (call);                                                               \
    if (_s != FL_OK) return _s;                                                    \
  } while (0)

#define FL_CHECK_ARG(cond, msg)                                                    \
  do {                                                                             \
    if (!(cond)) {                                                                 \
      ::fl::set_error("invalid argument: %s", msg);                                \
      return FL_ERR_ARG;                                                           \
    }                                                                              \
  } while (0)

// Grid sizes: a multiple of the SM count (152 on GB300) times resident CTAs.
int num_sms();
inline unsigned grid_for(int64_t n, int threads, int per_sm = 8) {
  int64_t b = (n + threads - 1) / threads;
  int64_t cap = (int64_t)num_sms() * per_sm;
  if (b > cap) b = cap;
  if (b < 1) b = 1;
  return (unsigned)b;
}

// Plain device buffer (cudaMalloc/cudaFree) with grow-only resize.
template <class T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  int reserve(size_t count) {
    if (count <= n && p) return FL_OK;
    release();
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      set_error("cudaMalloc(%zu bytes): %s", count * sizeof(T), cudaGetErrorString(e));
      return FL_ERR_NOMEM;
    }
    n = count;
    return FL_OK;
  }
};

// Device exclusive scan of int32 counts into int32 offsets (out[n] = total).
// Returns FL_ERR_ARG when the total does not fit in int32.
int exclusive_scan_i32(const int32_t* d_in, int32_t* d_out, int64_t n, cudaStream_t s);

// Device-wide error word written by kernels (bounded waits, pattern misses).
struct ErrWord {
  int32_t code;      // FL_OK or an FL_ERR_* status
  int32_t where;     // kernel-specific detail (element / row index)
};

// Graph-capturable FP64 CG on one system (batched solves).  cg_prepare may
// synchronise (first use of a mesh builds its sliced layout); the *_launch and
// cg_iterate calls only enqueue device work.
struct KrylovWork;
struct KspState;
struct SpArgs {
  int32_t n;
  const int32_t* findrm;
  const int32_t* colm;
  const double* val;
  const uint8_t* ghost;  // may be null
  KspState* st;
};

struct SellArgs {
  int32_t n;
  const int32_t* sptr;
  const int32_t* scol;
  const uint8_t* ghost;
  KspState* st;
  const int16_t* soff;  // column - row (2-byte indices) when not null; else scol
};

struct CgPlan {
  struct ::fl_mesh_t* m = nullptr;
  KrylovWork* W = nullptr;
  fl_solver_opts o{};
  const double* val = nullptr;
  const uint8_t* ghost = nullptr;
  const double* rhs = nullptr;
  double* x = nullptr;
  int n = 0, G = 2, np = 0;
  int ksp = 0, restart = 30;  // 0: CG (one iteration per cg_iterate), 1: GMRES (one cycle)
  unsigned gsp = 0, gv = 0, gsl = 0;
  int64_t sell_len = 0;
  const int32_t* smap = nullptr;
  SellArgs SA{};
  SpArgs A{};
};
int cg_prepare(CgPlan& P, struct ::fl_mesh_t* m, const fl_solver_opts* o, const double* val, const uint8_t* ghost,
               const double* rhs, double* x, cudaStream_t s);
void cg_setup_launch(CgPlan& P, cudaStream_t s);
void cg_iterate(CgPlan& P, cudaStream_t s);
void cg_finish_launch(CgPlan& P, cudaStream_t s);
int cg_report(CgPlan& P, fl_solve_report* rep, cudaStream_t s);
void cg_release(CgPlan& P);
KspState* cg_state(CgPlan& P);
void gather_done(KspState* const* d_states, int n, int* d_out, cudaStream_t s);
int csr_mult(struct ::fl_mesh_t* m, const double* val, const double* x, double* y, cudaStream_t s);

// Assembly pieces used by batches (no synchronisation, no allocation).
size_t assembly_scratch_doubles(const struct ::fl_mesh_t* m, const fl_advdif_params* p);
int assemble(struct ::fl_mesh_t* m, const fl_advdif_params* p, const fl_fields* f, double* val, double* rhs,
             cudaStream_t s, double* em_override, bool host_out = false);
int dirichlet_launch(struct ::fl_mesh_t* m, int32_t nb, const int32_t* nodes, int32_t base, const double* g,
                     const double* t, double dt, double* rhs, uint8_t* inactive, cudaStream_t s);
int autotune_assembly(struct ::fl_mesh_t* m, const fl_advdif_params* p, const fl_fields* f, double* val,
                      double* rhs, cudaStream_t s);
// Row pass of P1 FP64 element values in the symmetric coefficient-major layout
// em[k*E + e] (ten matrix entries, then four rhs entries per element).
int rows_p1_closed(struct ::fl_mesh_t* m, const double* em, double* val, double* rhs, cudaStream_t s);
// Row pass of P1 double-float row-slice records {K_a0, K_a1 | K_a2, r_a}
// (K_a3 from the zero row sum), 32 B per (element, local row).
int rows_p1_df(struct ::fl_mesh_t* m, const double* em, double* val, double* rhs, cudaStream_t s);

// Failure injection for tests of the bounded device waits (fl_set_wait_test):
// withhold >= 0 keeps one flag unset (colouring: that element never publishes
// its colour; fused P1 pass: that element-item group never counts complete);
// wait_ms > 0 bounds each wait to about that time instead of the defaults.
struct WaitTest {
  int32_t withhold = -1;
  double wait_ms = 0.0;
};
WaitTest& wait_test();

// node -> surface-face lists of the mesh (face_ptr / face_list: for every
// field node the faces holding it, ascending), from nf faces of floc nodes.
int node_face_lists(struct ::fl_mesh_t* m, int32_t nf, int32_t floc, const int32_t* faces, int32_t base,
                    cudaStream_t s);

// Per-translation-unit launch counters and workspace release hooks.
unsigned long long launches_mesh();
unsigned long long launches_assemble();
unsigned long long launches_krylov();
unsigned long long launches_gnn();
unsigned long long launches_amg();
unsigned long long launches_projection();
void release_krylov_work(struct ::fl_mesh_t* m);

}  // namespace fl

// Opaque mesh handle of the C-ABI: device mirrors of a field mesh and of its
// coordinate (topology) mesh, plus the cached sparsity and colouring that the
// reference caches in state / on the topology mesh.
struct fl_mesh_t {
  int device = 0;
  int32_t N = 0;     // field-mesh nodes (matrix rows)
  int32_t E = 0;     // elements
  int32_t loc = 0;   // nodes per element of the field mesh (4 or 10)
  int32_t Nx = 0;    // coordinate (P1 vertex) nodes
  int64_t nnz = 0;
  int32_t ncolours = 0;
  int32_t max_row = 0;  // longest CSR row
  // assembly tiles (set by the autotuner; results do not depend on them)
  int tile_elem_block = 256;  // threads per element-pass block
  int tile_elem_per_sm = 16;  // element-pass blocks per SM of the grid-stride grid
  int tile_rows = 1;          // row-pass tile index (see launch_rows); 3: fused P1 pass
  bool tuned = false;
  cudaStream_t stream = nullptr;

  fl::DevBuf<int32_t> ndglno;        // E*loc, 0-based, element-major
  fl::DevBuf<int32_t> xndglno;       // E*4
  fl::DevBuf<double> coords;         // 3*Nx
  fl::DevBuf<int32_t> ne_ptr, ne;    // field node -> (element<<4 | local) ascending
  fl::DevBuf<int32_t> ne_col;        // same incidences per node, ordered by element colour
  fl::DevBuf<uint32_t> ne_pos;       // per ne_col incidence: row position of each element node,
                                     // one byte per node, ceil(loc/4) words per incidence
  fl::DevBuf<int32_t> vne_ptr, vne;  // vertex -> element ascending
  fl::DevBuf<int32_t> findrm, colm, centrm;
  fl::DevBuf<int32_t> colour;        // E, 1-based
  fl::DevBuf<int32_t> colour_elems;  // E, sorted by (colour, element)
  std::vector<int32_t> colour_ptr;   // ncolours+1 (host)
  fl::DevBuf<fl::ErrWord> err;       // 1 word
  fl::DevBuf<int32_t> tpos;          // per entry (k, j): position of (j, k) (built on first use)
  // fused P1 element + row pass (built on first use)
  int fz_state = 0;                  // 0 not built, 1 built, -1 not applicable
  int32_t fz_nitems = 0;
  fl::DevBuf<int32_t> fz_perm, fz_rec, fz_items, fz_need, fz_ctl;
  // pipelined P1 assembly into pinned host arrays (built with the fused plan):
  // row chunk k = rows [ck_rows[k], ck_rows[k+1]) needs the records at element
  // positions below ck_elem[k+1], which read field values below ck_node[k+1];
  // its entries are val[ck_val[k], ck_val[k+1])
  std::vector<int32_t> ck_rows, ck_elem, ck_node;
  std::vector<int64_t> ck_val;
  // copy stream (field uploads, result copies) and row-pass stream
  cudaStream_t ck_streams[2] = {nullptr, nullptr};
  std::vector<cudaEvent_t> ck_ev;  // per chunk: rows written, fields uploaded, records written
  struct fl_mesh_t* so_parent = nullptr;  // second-order pattern handles: the mesh they square
  // second-order handles of a rectangular factor C (fl_gpu_rect_secondorder_register): the handle
  // holding C's pattern, and C's pattern transposed (column -> rows, ascending) with the position
  // of every transposed entry in C
  struct fl_mesh_t* a_pat = nullptr;
  fl::DevBuf<int32_t> tr_ptr, tr_col, tr_pos;
  fl::DevBuf<float2> bt;                  // second-order handles: transposed product operand
  fl::DevBuf<int32_t> pair_off;           // second-order handles: pairs of each first-order entry
  fl::DevBuf<uint8_t> pair_map;           // second-order handles: output slot of every pair
  fl::DevBuf<int32_t> face_cnt, face_ptr, face_list;  // node -> surface faces (divergence surface terms)
  fl::DevBuf<double> em;             // element matrices + rhs (coefficient-major scratch)
  // staging buffers of the host-pointer entry points (grow-only)
  fl::DevBuf<double> st_val, st_rhs, st_t, st_u, st_src, st_abs, st_x, st_g;
  fl::DevBuf<uint8_t> st_ina;
  fl::DevBuf<int32_t> st_nodes;
  // element-kernel timing of the last assembly (fl_set_kernel_timing)
  bool timing = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool timed = false;
};
