// fl_projection.cu -- the pressure-projection matrices of a P1 velocity /
// P1 pressure discretisation on one mesh:
//   * the divergence matrix C^T and the lumped masses of
//     assemble_divergence_matrix_cg (assemble/Divergence_Matrix_CG.F90:67-375),
//     including the surface terms of the integrated-by-parts form;
//   * the lumped mass of compute_lumped_mass (femtools/FEFields.F90:161-214);
//   * the second-order sparsity of get_csr_sparsity_secondorder
//     (femtools/Sparsity_Patterns_Meshes.F90:122-148 -> make_sparsity_transpose,
//     femtools/Sparsity_Patterns.F90:87-148), bit-exact;
//   * the weighted row products mult_div_vector_div_T and
//     mult_div_invscalar_div_T (femtools/Sparse_Matrices_Fields.F90:590-748)
//     that form C M_l^-1 C^T (assemble_masslumped_cmc,
//     assemble/Assemble_CMC.F90:119-135) and the P1-P1 stabilisation
//     K M^-1 K (assemble_kmk_matrix, assemble/Momentum_CG.F90:2707-2766);
//   * the mass-lumped projection right-hand side and velocity correction
//     (assemble_masslumped_poisson_rhs, correct_masslumped_velocity,
//     assemble/Momentum_CG.F90:2544-2575,2670-2705).
//
// Layout.  C^T is the reference's block_csr_matrix with blocks (1, dim): three
// FP64 value arrays over the mesh's first-order pattern.  Vector fields are
// vector_field%val(3, N): x, y, z of a node adjacent.  The second-order
// pattern is a pattern-only handle whose parent is the mesh; the products
// read the parent's pattern and its transpose map tpos (tpos[p] = position of
// (colm[p], row) for the entry p of a row: the pattern is structurally
// symmetric).
//
// Kernels.
//   k_div_elem   element pass: per element the nine signed cofactors / 24 and
//                |det| / 24 (the whole P1 element matrix: row a of
//                shape_dshape is sign(det) cof(:, b) / 24 for every b), as
//                double-float pairs, 80 B, written through shared memory
//                with coalesced stores.
//   k_div_rows   row pass: one thread per row sums its incidences in colour
//                order (deterministic) into double-float shared accumulators.
//   k_div_faces  surface terms, one thread per boundary node, faces in
//                ascending order after the element terms.
//   k_so_rows    second-order pattern: one warp per row gathers the rows of
//                its neighbours, sorts them bitonically in shared memory and
//                keeps the distinct columns.
//   k_bt_gather  b transposed along the pattern rows (through tpos), as
//                double-float pairs: the product's loads of b are coalesced.
//   k_rowprod    out(i,j) = sum_k sum_d a_d(i,k) w_d(k) b_d(j,k): one warp per
//                output row, the row's columns and double-float accumulators
//                in shared memory; the two half-warps take two k at a time and
//                add in a fixed order, so every sum is deterministic.
//   k_kmk_elem   P1 pressure-diffusion element matrix
//                0.5 V grad N^T h_bar grad N with h_bar the element's edge-
//                length tensor (closed form below), in double-float, written
//                as the P1 assembly's row-slice records and summed by its
//                double-float row pass.
#include <algorithm>
#include <cfloat>
#include <climits>
#include <cmath>
#include <vector>

#include "fl_internal.cuh"
#include "fl_device.cuh"
#include "fl_df64.cuh"
#include "fl_refelem.h"

namespace fl {

unsigned long long launches_projection() { return unit_launches(); }

namespace {

constexpr int kT = 256;

cudaStream_t pick(fl_mesh_t* m, void* stream) { return stream ? (cudaStream_t)stream : m->stream; }

// ------------------------------------------------------------- divergence --
struct DivElemArgs {
  int32_t E;
  const int32_t* xnd;
  const double* X;
  float4* rec;  // 5 float4 per element
  df k24;       // 1/24
};

__global__ void __launch_bounds__(256) k_div_elem(DivElemArgs A) {
  note_launch();
  extern __shared__ float4 stage_all[];
  const int lane = threadIdx.x & 31;
  float4* stage = stage_all + (threadIdx.x >> 5) * 160;
  for (int base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < A.E; base += gridDim.x * blockDim.x) {
    const int e = base + lane;
    if (e < A.E) {
      const int4 v = __ldg(reinterpret_cast<const int4*>(A.xnd) + e);
      const int vi[4] = {v.x, v.y, v.z, v.w};
      double x[4][3];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int a = 0; a < 3; ++a) x[i][a] = __ldg(A.X + (uint32_t)(3 * vi[i] + a));
      df J[3][3];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) J[a][b] = df_from_double(x[b][a] - x[3][a]);
      df c[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, k1 = (k + 1) % 3, k2 = (k + 2) % 3;
          c[i][k] = df_mul_sub_mul(J[i1][k1], J[i2][k2], J[i2][k1], J[i1][k2]);
        }
      const df det = df_dot3(J[0][0], c[0][0], J[1][0], c[1][0], J[2][0], c[2][0]);
      const df s = det.hi < 0.0f ? df_neg(A.k24) : A.k24;
      df r[10];
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int b = 0; b < 3; ++b) r[3 * d + b] = df_mul(c[d][b], s);
      r[9] = df_mul(df_abs(det), A.k24);
      float4* o = stage + lane * 5;
#pragma unroll
      for (int k = 0; k < 5; ++k) o[k] = make_float4(r[2 * k].hi, r[2 * k].lo, r[2 * k + 1].hi, r[2 * k + 1].lo);
    }
    __syncwarp();
    float4* out = A.rec + (uint32_t)base * 5u;
    const int nvalid = min(32, A.E - base) * 5;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const int idx = k * 32 + lane;
      if (idx < nvalid) out[idx] = stage[idx];
    }
    __syncwarp();
  }
}

struct DivRowArgs {
  int32_t N;
  const int32_t* ne_ptr;
  const int32_t* ne_col;
  const uint32_t* ne_pos;
  const int32_t* findrm;
  const float4* rec;
  double* ct0;
  double* ct1;
  double* ct2;
  double* ct_rhs;  // zeroed when given
  double* dml;
  double* gml;
};

__device__ __forceinline__ df f2(float x, float y) { return {x, y}; }

// CT: assemble the three blocks; BYPARTS: -dshape_shape instead of shape_dshape.
template <int THREADS, int RMAX, bool CT, bool BYPARTS>
__global__ void __launch_bounds__(THREADS) k_div_rows(DivRowArgs P) {
  note_launch();
  extern __shared__ unsigned char smem_raw[];
  float2* acc = reinterpret_cast<float2*>(smem_raw);  // [3][RMAX][THREADS]
  const int t = threadIdx.x;
  double* ct[3] = {P.ct0, P.ct1, P.ct2};
  for (int row = blockIdx.x * THREADS + t; row < P.N; row += gridDim.x * THREADS) {
    const int base = __ldg(P.findrm + row), L = __ldg(P.findrm + row + 1) - base;
    const bool in_smem = L <= RMAX;
    if (CT) {
      if (in_smem) {
        for (int d = 0; d < 3; ++d)
          for (int k = 0; k < L; ++k) acc[(d * RMAX + k) * THREADS + t] = make_float2(0.0f, 0.0f);
      } else {
        for (int d = 0; d < 3; ++d)
          for (int k = 0; k < L; ++k) ct[d][base + k] = 0.0;
      }
    }
    df mass = {0.0f, 0.0f};
    const int ib = __ldg(P.ne_ptr + row), ie = __ldg(P.ne_ptr + row + 1);
    for (int q = ib; q < ie; ++q) {
      const int inc = __ldg(P.ne_col + q);
      const int e = inc >> 4, a = inc & 15;
      const float4* r = P.rec + (uint32_t)e * 5u;
      const float4 r4 = __ldg(r + 4);
      mass = df_add(mass, f2(r4.z, r4.w));
      if (!CT) continue;
      const uint32_t pw = __ldg(P.ne_pos + q);
      const float4 r0 = __ldg(r), r1 = __ldg(r + 1), r2 = __ldg(r + 2), r3 = __ldg(r + 3);
      df c[3][4];
      c[0][0] = f2(r0.x, r0.y); c[0][1] = f2(r0.z, r0.w); c[0][2] = f2(r1.x, r1.y);
      c[1][0] = f2(r1.z, r1.w); c[1][1] = f2(r2.x, r2.y); c[1][2] = f2(r2.z, r2.w);
      c[2][0] = f2(r3.x, r3.y); c[2][1] = f2(r3.z, r3.w); c[2][2] = f2(r4.x, r4.y);
#pragma unroll
      for (int d = 0; d < 3; ++d) c[d][3] = df_neg(df_add(df_add(c[d][0], c[d][1]), c[d][2]));
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        df own = c[d][0];
        if (BYPARTS) {
          own = a == 1 ? c[d][1] : own;
          own = a == 2 ? c[d][2] : own;
          own = a == 3 ? c[d][3] : own;
          own = df_neg(own);
        }
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const df v = BYPARTS ? own : c[d][b];
          const int pos = (pw >> (8 * b)) & 0xffu;
          if (in_smem) {
            float2* p = &acc[(d * RMAX + pos) * THREADS + t];
            const df sum = df_add(f2(p->x, p->y), v);
            *p = make_float2(sum.hi, sum.lo);
          } else {
            ct[d][base + pos] += df_to_double(v);
          }
        }
      }
    }
    if (CT && in_smem)
      for (int d = 0; d < 3; ++d)
        for (int k = 0; k < L; ++k) {
          const float2 v = acc[(d * RMAX + k) * THREADS + t];
          ct[d][base + k] = df_to_double(f2(v.x, v.y));
        }
    const double ms = df_to_double(mass);
    if (P.dml) P.dml[row] = ms;
    if (P.gml) P.gml[row] = ms;
    if (P.ct_rhs) P.ct_rhs[row] = 0.0;
  }
}

// node -> surface faces incidence (counting sort, lists sorted ascending);
// faces hold floc nodes each
__global__ void k_face_count(int32_t nf, int32_t floc, const int32_t* __restrict__ faces, int32_t base, int32_t N,
                             int32_t* __restrict__ cnt, ErrWord* err) {
  note_launch();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < (int64_t)floc * nf;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int v = faces[k] - base;
    if (v < 0 || v >= N) {
      set_err(err, FL_ERR_ARG, (int)(k / floc));
      continue;
    }
    atomicAdd(cnt + v, 1);
  }
}

__global__ void k_face_fill(int32_t nf, int32_t floc, const int32_t* __restrict__ faces, int32_t base, int32_t N,
                            const int32_t* __restrict__ fptr, int32_t* __restrict__ fill,
                            int32_t* __restrict__ flist) {
  note_launch();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < (int64_t)floc * nf;
       k += (int64_t)gridDim.x * blockDim.x) {
    const int v = faces[k] - base;
    if (v < 0 || v >= N) continue;
    const int slot = atomicAdd(fill + v, 1);
    flist[fptr[v] + slot] = (int)(k / floc);
  }
}

__global__ void k_face_sort(int32_t N, const int32_t* __restrict__ fptr, int32_t* __restrict__ flist) {
  note_launch();
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) {
    const int b = fptr[v], e = fptr[v + 1];
    for (int i = b + 1; i < e; ++i) {
      const int x = flist[i];
      int j = i - 1;
      while (j >= b && flist[j] > x) {
        flist[j + 1] = flist[j];
        --j;
      }
      flist[j + 1] = x;
    }
  }
}

struct FaceArgs {
  int32_t N;
  int32_t base;
  const int32_t* fptr;
  const int32_t* flist;
  const int32_t* faces;
  const int32_t* face_ele;
  const int32_t* bc_type;
  const double* bc_val;
  const int32_t* xnd;
  const double* X;
  const int32_t* findrm;
  const int32_t* colm;
  double* ct0;
  double* ct1;
  double* ct2;
  double* ct_rhs;
  int32_t E;
  ErrWord* err;
};

// Surface terms of the integrated-by-parts divergence (Divergence_Matrix_CG.F90
// :312-366).  Face mass of a P1 triangle: detJ/12 on the diagonal and detJ/24
// off it (the three-point rule is exact for it); normal = facet_normal
// (Transform_elements.F90:1527-1553).
__global__ void k_div_faces(FaceArgs F) {
  note_launch();
  double* ct[3] = {F.ct0, F.ct1, F.ct2};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < F.N; i += gridDim.x * blockDim.x) {
    const int qb = F.fptr[i], qe = F.fptr[i + 1];
    for (int q = qb; q < qe; ++q) {
      const int f = F.flist[q];
      int ty[3];
      bool skip = false;
      for (int d = 0; d < 3; ++d) {
        ty[d] = F.bc_type ? F.bc_type[3 * f + d] : 0;
        skip = skip || ty[d] == 2 || ty[d] == 3 || ty[d] == 4;
      }
      if (skip) continue;
      int fn[3], li = -1;
      for (int j = 0; j < 3; ++j) {
        fn[j] = F.faces[3 * f + j] - F.base;
        if (fn[j] == i) li = j;
      }
      const int el = F.face_ele[f] - F.base;
      if (li < 0 || el < 0 || el >= F.E) {
        set_err(F.err, FL_ERR_ARG, f);
        continue;
      }
      double Xf[3][3], cf[3] = {0.0, 0.0, 0.0}, ce[3] = {0.0, 0.0, 0.0};
      for (int j = 0; j < 3; ++j)
        for (int a = 0; a < 3; ++a) {
          Xf[j][a] = F.X[3 * fn[j] + a];
          cf[a] += Xf[j][a];
        }
      for (int j = 0; j < 4; ++j) {
        const int v = F.xnd[4 * el + j];
        for (int a = 0; a < 3; ++a) ce[a] += F.X[3 * v + a];
      }
      double J0[3], J1[3], ow[3];
      for (int a = 0; a < 3; ++a) {
        J0[a] = Xf[0][a] - Xf[2][a];
        J1[a] = Xf[1][a] - Xf[2][a];
        ow[a] = cf[a] / 3.0 - ce[a] / 4.0;
      }
      double n[3] = {J0[1] * J1[2] - J0[2] * J1[1], J0[2] * J1[0] - J0[0] * J1[2], J0[0] * J1[1] - J0[1] * J1[0]};
      const double detJ = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      const double o = n[0] * ow[0] + n[1] * ow[1] + n[2] * ow[2];
      for (int a = 0; a < 3; ++a) n[a] *= o;
      const double len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      for (int a = 0; a < 3; ++a) n[a] /= len;
      double mrow[3];
      for (int j = 0; j < 3; ++j) mrow[j] = detJ * (j == li ? 1.0 / 12.0 : 1.0 / 24.0);
      const double* bv = F.bc_val ? F.bc_val + 9 * f : nullptr;
      if (ty[0] == 5 && F.ct_rhs) {
        if (!bv) {
          set_err(F.err, FL_ERR_ARG, f);
          continue;
        }
        double r = 0.0;
        for (int j = 0; j < 3; ++j) r += mrow[j] * bv[3 * j];
        F.ct_rhs[i] -= r;
        continue;
      }
      const int rb = F.findrm[i], re = F.findrm[i + 1];
      for (int d = 0; d < 3; ++d) {
        if (ty[d] == 1 && F.ct_rhs) {
          if (!bv) {
            set_err(F.err, FL_ERR_ARG, f);
            continue;
          }
          double r = 0.0;
          for (int j = 0; j < 3; ++j) r += n[d] * mrow[j] * bv[3 * j + d];
          F.ct_rhs[i] -= r;
        } else {
          for (int j = 0; j < 3; ++j) {
            const int p = csr_find(F.colm, rb, re, fn[j]);
            if (p < 0) {
              set_err(F.err, FL_ERR_OUTSIDE_PATTERN, i);
              continue;
            }
            ct[d][p] += n[d] * mrow[j];
          }
        }
      }
    }
  }
}

// Surface terms of the integrated-by-parts Taylor-Hood divergence (the same
// loop, Divergence_Matrix_CG.F90:312-366, with P1 pressure test functions and
// P2 velocity field functions on each face): one thread per pressure row,
// its faces in ascending order.  The face integrals are detJ T(i, j) with
// T(i, j) = sum_g w_g L_i N_j over the triangle rule (P1 x P2, computed on
// the host), normal = facet_normal as in k_div_faces.
struct ThFaceArgs {
  FaceArgs F;          // faces = pressure (vertex) nodes; findrm / colm = the rectangular pattern
  const int32_t* vfaces;  // six P2 velocity nodes per face
  double T[3][6];
};

__global__ void k_div_faces_th(ThFaceArgs A) {
  note_launch();
  const FaceArgs& F = A.F;
  double* ct[3] = {F.ct0, F.ct1, F.ct2};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < F.N; i += gridDim.x * blockDim.x) {
    const int qb = F.fptr[i], qe = F.fptr[i + 1];
    for (int q = qb; q < qe; ++q) {
      const int f = F.flist[q];
      int ty[3];
      bool skip = false;
      for (int d = 0; d < 3; ++d) {
        ty[d] = F.bc_type ? F.bc_type[3 * f + d] : 0;
        skip = skip || ty[d] == 2 || ty[d] == 3 || ty[d] == 4;
      }
      if (skip) continue;
      int fn[3], li = -1;
      for (int j = 0; j < 3; ++j) {
        fn[j] = F.faces[3 * f + j] - F.base;
        if (fn[j] == i) li = j;
      }
      const int el = F.face_ele[f] - F.base;
      if (li < 0 || el < 0 || el >= F.E) {
        set_err(F.err, FL_ERR_ARG, f);
        continue;
      }
      double Xf[3][3], cf[3] = {0.0, 0.0, 0.0}, ce[3] = {0.0, 0.0, 0.0};
      for (int j = 0; j < 3; ++j)
        for (int a = 0; a < 3; ++a) {
          Xf[j][a] = F.X[3 * fn[j] + a];
          cf[a] += Xf[j][a];
        }
      for (int j = 0; j < 4; ++j) {
        const int v = F.xnd[4 * el + j];
        for (int a = 0; a < 3; ++a) ce[a] += F.X[3 * v + a];
      }
      double J0[3], J1[3], ow[3];
      for (int a = 0; a < 3; ++a) {
        J0[a] = Xf[0][a] - Xf[2][a];
        J1[a] = Xf[1][a] - Xf[2][a];
        ow[a] = cf[a] / 3.0 - ce[a] / 4.0;
      }
      double n[3] = {J0[1] * J1[2] - J0[2] * J1[1], J0[2] * J1[0] - J0[0] * J1[2], J0[0] * J1[1] - J0[1] * J1[0]};
      const double detJ = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      const double o = n[0] * ow[0] + n[1] * ow[1] + n[2] * ow[2];
      for (int a = 0; a < 3; ++a) n[a] *= o;
      const double len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      for (int a = 0; a < 3; ++a) n[a] /= len;
      double mrow[6];
      for (int j = 0; j < 6; ++j) mrow[j] = detJ * A.T[li][j];
      const double* bv = F.bc_val ? F.bc_val + 18 * (int64_t)f : nullptr;
      if (ty[0] == 5 && F.ct_rhs) {
        if (!bv) {
          set_err(F.err, FL_ERR_ARG, f);
          continue;
        }
        double r = 0.0;
        for (int j = 0; j < 6; ++j) r += mrow[j] * bv[3 * j];
        F.ct_rhs[i] -= r;
        continue;
      }
      int vn[6];
      for (int j = 0; j < 6; ++j) vn[j] = A.vfaces[6 * f + j] - F.base;
      const int rb = F.findrm[i], re = F.findrm[i + 1];
      for (int d = 0; d < 3; ++d) {
        if (ty[d] == 1 && F.ct_rhs) {
          if (!bv) {
            set_err(F.err, FL_ERR_ARG, f);
            continue;
          }
          double r = 0.0;
          for (int j = 0; j < 6; ++j) r += n[d] * mrow[j] * bv[3 * j + d];
          F.ct_rhs[i] -= r;
        } else {
          for (int j = 0; j < 6; ++j) {
            const int p = csr_find(F.colm, rb, re, vn[j]);
            if (p < 0) {
              set_err(F.err, FL_ERR_OUTSIDE_PATTERN, i);
              continue;
            }
            ct[d][p] += n[d] * mrow[j];
          }
        }
      }
    }
  }
}

// ------------------------------------------------------- pattern products --
// tpos[p] for the entry p = (k, j) of row k: the position of (j, k) in row j.
__global__ void k_tpos(int32_t N, const int32_t* __restrict__ findrm, const int32_t* __restrict__ colm,
                       int32_t* __restrict__ tpos, ErrWord* err) {
  note_launch();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x)
    for (int p = findrm[k]; p < findrm[k + 1]; ++p) {
      const int j = colm[p];
      const int t = csr_find(colm, findrm[j], findrm[j + 1], k);
      if (t < 0) set_err(err, FL_ERR_ARG, k);
      tpos[p] = t < 0 ? p : t;
    }
}

constexpr int kSoWarps = 4;
constexpr int kSoCap = 1024;  // gathered candidates of one row

// pass 0: distinct-column count of every row (and the longest row);
// pass 1: the columns, ascending, and the diagonal position.
__global__ void __launch_bounds__(kSoWarps * 32) k_so_rows(int32_t N, const int32_t* __restrict__ fr,
                                                          const int32_t* __restrict__ cm,
                                                          const int32_t* __restrict__ tr,
                                                          const int32_t* __restrict__ tc,
                                                          const int32_t* __restrict__ optr,
                                                          int32_t* __restrict__ cnt, int32_t* __restrict__ ocol,
                                                          int32_t* __restrict__ ocentre, int32_t* maxrow,
                                                          ErrWord* err, int pass) {
  note_launch();
  __shared__ int32_t keys_all[kSoWarps][kSoCap];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int32_t* keys = keys_all[w];
  for (int row = blockIdx.x * kSoWarps + w; row < N; row += gridDim.x * kSoWarps) {
    int nc = 0;
    const int qb = fr[row], qe = fr[row + 1];
    for (int q = qb; q < qe; ++q) {
      const int k = cm[q];
      const int kb = tr[k], len = tr[k + 1] - kb;
      for (int t = lane; t < len; t += 32)
        if (nc + t < kSoCap) keys[nc + t] = tc[kb + t];
      nc += len;
    }
    if (nc > kSoCap) {
      if (lane == 0) set_err(err, FL_ERR_UNSUPPORTED, row);
      __syncwarp();
      continue;
    }
    int pw = 1;
    while (pw < nc) pw <<= 1;
    for (int t = nc + lane; t < pw; t += 32) keys[t] = INT_MAX;
    __syncwarp();
    for (int size = 2; size <= pw; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int t = lane; t < pw; t += 32) {
          const int l = t ^ stride;
          if (l > t) {
            const int a = keys[t], b = keys[l];
            const bool up = (t & size) == 0;
            if ((a > b) == up) {
              keys[t] = b;
              keys[l] = a;
            }
          }
        }
        __syncwarp();
      }
    int total = 0;
    const int o0 = pass ? optr[row] : 0;
    for (int t0 = 0; t0 < nc; t0 += 32) {
      const int t = t0 + lane;
      const bool head = t < nc && (t == 0 || keys[t] != keys[t - 1]);
      const unsigned hm = __ballot_sync(0xffffffffu, head);
      if (pass && head) {
        const int slot = total + __popc(hm & ((1u << lane) - 1u));
        ocol[o0 + slot] = keys[t];
        if (keys[t] == row) ocentre[row] = o0 + slot;
      }
      total += __popc(hm);
    }
    if (pass == 0 && lane == 0) {
      cnt[row] = total;
      atomicMax(maxrow, total);
    }
    __syncwarp();
  }
}

constexpr int kPW = 8;      // warps per block of the product kernel (two rows per warp)
constexpr int kPCap = 192;  // longest output row held in shared memory

// bt[d][r] = b_d(j, k) for the entry r = (k, j) of row k: B transposed along
// the pattern's rows (a gather through tpos), as double-float pairs, so that
// the product reads it with coalesced loads.
template <int NDIM>
__global__ void k_bt_gather(int64_t nnz, const int32_t* __restrict__ tpos, const double* __restrict__ b0,
                            const double* __restrict__ b1, const double* __restrict__ b2, float2* __restrict__ bt) {
  note_launch();
  for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nnz; r += (int64_t)gridDim.x * blockDim.x) {
    const int t = __ldg(tpos + r);
    const double* b[3] = {b0, b1, b2};
#pragma unroll
    for (int d = 0; d < NDIM; ++d) {
      const df x = df_from_double(__ldg(b[d] + t));
      bt[d * nnz + r] = make_float2(x.hi, x.lo);
    }
  }
}

// Slot map of the row products: for the entry q = (i, k) of the first-order
// pattern and the t-th entry (k, j) of row k, the position of j in output row
// i, one byte per pair at pmap[poff[q] + t] (output rows hold at most kPCap
// entries).  Built once per second-order pattern.
__global__ void k_pair_count(int32_t N, const int32_t* __restrict__ fr, const int32_t* __restrict__ cm,
                             const int32_t* __restrict__ tr, int32_t* __restrict__ cnt) {
  note_launch();
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < fr[N]; q += gridDim.x * blockDim.x) {
    const int k = cm[q];
    cnt[q] = tr[k + 1] - tr[k];
  }
}

__global__ void k_pair_map(int32_t N, const int32_t* __restrict__ fr, const int32_t* __restrict__ cm,
                           const int32_t* __restrict__ tr, const int32_t* __restrict__ tc,
                           const int32_t* __restrict__ optr, const int32_t* __restrict__ ocol,
                           const int32_t* __restrict__ poff, uint8_t* __restrict__ pmap, ErrWord* err) {
  note_launch();
  const int lane = threadIdx.x & 31;
  const int nw = gridDim.x * (blockDim.x >> 5);
  for (int i = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); i < N; i += nw) {
    const int ob = optr[i], L = optr[i + 1] - ob;
    if (L > kPCap) {
      if (lane == 0) set_err(err, FL_ERR_UNSUPPORTED, i);
      continue;
    }
    for (int q = fr[i]; q < fr[i + 1]; ++q) {
      const int k = cm[q], kb = tr[k], len = tr[k + 1] - kb;
      for (int t = lane; t < len; t += 32) {
        const int j = tc[kb + t];
        int lo = 0, hi = L;
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (ocol[ob + mid] < j) lo = mid + 1;
          else hi = mid;
        }
        if (lo >= L || ocol[ob + lo] != j) set_err(err, FL_ERR_OUTSIDE_PATTERN, i);
        pmap[(int64_t)poff[q] + t] = (uint8_t)(lo < L ? lo : 0);
      }
    }
  }
}

struct RowProdArgs {
  int32_t n;
  int64_t annz;
  const int32_t* aptr;
  const int32_t* acol;
  const int32_t* tptr;  // the second factor's rows: aptr for a square symmetric pattern
  const int32_t* optr;
  const int32_t* poff;   // per first-order entry (i, k): start of its pairs in pmap
  const uint8_t* pmap;   // output slot of every pair
  const double* a[3];
  const float2* bt;  // NDIM blocks of annz pairs
  const double* w;   // NDIM values per node; the divisor s when DIV
  double theta;      // DIV: the divisor is theta * s when scale != 0
  int scale;
  double* out;
  ErrWord* err;
};

// Double-float arithmetic on the FP32 pipes (GB300's FP64 rate is 1/60 of
// FP32).  One half-warp per output row i (two rows per warp).  The k of row
// i go in groups of 16: each lane loads one k's data (column k, the extent and
// pair offset of row k, c_d = a_d(i,k) w_d(k) or a(i,k) / s(k)) into shared
// memory, then the half-warp walks the group's k in ascending order, reading
// each k's data as a shared-memory broadcast.  In step k, lane t owns entry t
// of row k, (k, j), and adds c . bt(k, j) to the slot of j in the output row
// (shared memory, double-float); the k are added one after the other, so
// every sum has a fixed order.  The step has no branch: lanes past the end of
// row k read the first entry and add into a dummy slot.  A group holding a
// row k longer than 16 entries takes the general loop over its entries in
// runs of 16.
template <int NDIM, bool DIV>
__global__ void __launch_bounds__(kPW * 32, 4) k_rowprod(RowProdArgs P) {
  note_launch();
  __shared__ float2 s_acc_all[2 * kPW][kPCap + 1];  // + one dummy slot
  __shared__ int4 s_k_all[2 * kPW][16];              // {row start, extent, pair offset, -}
  __shared__ float2 s_c_all[2 * kPW][NDIM][16];
  const int lane = threadIdx.x & 31, half = lane >> 4, hl = lane & 15;
  const int hw = (threadIdx.x >> 5) * 2 + half;  // half-warp index in the block
  float2* s_acc = s_acc_all[hw];
  int4* s_k = s_k_all[hw];
  float2 (*s_c)[16] = s_c_all[hw];
  const float2* bt[NDIM];
#pragma unroll
  for (int d = 0; d < NDIM; ++d) bt[d] = P.bt + d * P.annz;
  const int nrow_steps = (P.n + 2 * kPW * gridDim.x - 1) / (2 * kPW * gridDim.x);
  for (int it = 0; it < nrow_steps; ++it) {
    const int row = (it * gridDim.x + blockIdx.x) * 2 * kPW + hw;
    const bool live = row < P.n;
    int ob = 0, L = 0, qb = 0, qe = 0;
    if (live) {
      ob = __ldg(P.optr + row);
      L = __ldg(P.optr + row + 1) - ob;
      qb = __ldg(P.aptr + row);
      qe = __ldg(P.aptr + row + 1);
    }
    if (L > kPCap) {  // the map build rejects such patterns
      L = 0;
      qe = qb;
    }
    for (int t = hl; t < L; t += 16) s_acc[t] = make_float2(0.0f, 0.0f);
    __syncwarp();
    // both halves run the same number of k steps (the longer row's)
    const int nk = qe - qb;
    const int nk_max = max(nk, __shfl_xor_sync(0xffffffffu, nk, 16));
    for (int g0 = 0; g0 < nk_max; g0 += 16) {
      // this group's k data, one k per lane, into shared memory
      const int qg = qb + g0 + hl;
      int kb = 0, klen = 0, po = 0;
      df c[NDIM];
#pragma unroll
      for (int d = 0; d < NDIM; ++d) c[d] = {0.0f, 0.0f};
      if (qg < qe) {
        const int k = __ldg(P.acol + qg);
        kb = __ldg(P.tptr + k);
        klen = __ldg(P.tptr + k + 1) - kb;
        po = __ldg(P.poff + qg);
        if (DIV) {
          double sk = __ldg(P.w + k);
          if (P.scale) sk = sk * P.theta;
          c[0] = df_mul(df_from_double(__ldg(P.a[0] + qg)), df_rcp(df_from_double(sk)));
        } else {
#pragma unroll
          for (int d = 0; d < NDIM; ++d)
            c[d] = df_mul(df_from_double(__ldg(P.a[d] + qg)), df_from_double(__ldg(P.w + NDIM * k + d)));
        }
      }
      s_k[hl] = make_int4(kb, klen, po, 0);
#pragma unroll
      for (int d = 0; d < NDIM; ++d) s_c[d][hl] = make_float2(c[d].hi, c[d].lo);
      int lmax = klen;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
      __syncwarp();
      const int gn = min(16, nk_max - g0);
      if (lmax <= 16) {
        // step u's slot and operands are loaded during step u-1's arithmetic
        int slot;
        float2 b[NDIM];
        {
          const int4 kk = s_k[0];
          const bool ok = hl < kk.y;
          slot = ok ? (int)__ldg(P.pmap + kk.z + hl) : kPCap;
          const int idx = kk.x + (ok ? hl : 0);
#pragma unroll
          for (int d = 0; d < NDIM; ++d) b[d] = __ldg(bt[d] + idx);
        }
        for (int u = 0; u < gn; ++u) {
          int nslot = kPCap;
          float2 nb[NDIM];
#pragma unroll
          for (int d = 0; d < NDIM; ++d) nb[d] = b[d];
          if (u + 1 < gn) {
            const int4 kk = s_k[u + 1];
            const bool ok = hl < kk.y;
            nslot = ok ? (int)__ldg(P.pmap + kk.z + hl) : kPCap;
            const int idx = kk.x + (ok ? hl : 0);
#pragma unroll
            for (int d = 0; d < NDIM; ++d) nb[d] = __ldg(bt[d] + idx);
          }
          df v;
          if (NDIM == 3) {
            const float2 c0 = s_c[0][u], c1 = s_c[NDIM > 1 ? 1 : 0][u], c2 = s_c[NDIM > 2 ? 2 : 0][u];
            v = df_dot3({c0.x, c0.y}, {b[0].x, b[0].y}, {c1.x, c1.y}, {b[NDIM > 1 ? 1 : 0].x, b[NDIM > 1 ? 1 : 0].y},
                        {c2.x, c2.y}, {b[NDIM > 2 ? 2 : 0].x, b[NDIM > 2 ? 2 : 0].y});
          } else {
            const float2 c0 = s_c[0][u];
            v = df_mul({c0.x, c0.y}, {b[0].x, b[0].y});
#pragma unroll
            for (int d = 1; d < NDIM; ++d) {
              const float2 cd = s_c[d][u];
              v = df_add(v, df_mul({cd.x, cd.y}, {b[d].x, b[d].y}));
            }
          }
          const float2 o = s_acc[slot];
          const df sum = df_add({o.x, o.y}, v);
          s_acc[slot] = make_float2(sum.hi, sum.lo);
          __syncwarp();  // the next k may add to the same slots from other lanes
          slot = nslot;
#pragma unroll
          for (int d = 0; d < NDIM; ++d) b[d] = nb[d];
        }
      } else {
        for (int u = 0; u < gn; ++u) {
          const int4 kk = s_k[u];
          df cu[NDIM];
#pragma unroll
          for (int d = 0; d < NDIM; ++d) cu[d] = {s_c[d][u].x, s_c[d][u].y};
          for (int m0 = 0; m0 < kk.y; m0 += 16) {
            const int e = m0 + hl;
            if (e < kk.y) {
              const int sl = __ldg(P.pmap + kk.z + e);
              df v;
              if (NDIM == 3) {
                const float2 b0 = __ldg(bt[0] + kk.x + e), b1 = __ldg(bt[NDIM > 1 ? 1 : 0] + kk.x + e),
                             b2 = __ldg(bt[NDIM > 2 ? 2 : 0] + kk.x + e);
                v = df_dot3(cu[0], {b0.x, b0.y}, cu[NDIM > 1 ? 1 : 0], {b1.x, b1.y}, cu[NDIM > 2 ? 2 : 0],
                            {b2.x, b2.y});
              } else {
                const float2 b0 = __ldg(bt[0] + kk.x + e);
                v = df_mul(cu[0], {b0.x, b0.y});
#pragma unroll
                for (int d = 1; d < NDIM; ++d) {
                  const float2 bd = __ldg(bt[d] + kk.x + e);
                  v = df_add(v, df_mul(cu[d], {bd.x, bd.y}));
                }
              }
              const float2 o = s_acc[sl];
              const df sum = df_add({o.x, o.y}, v);
              s_acc[sl] = make_float2(sum.hi, sum.lo);
            }
            __syncwarp(0xffffu << (half * 16));
          }
        }
      }
      __syncwarp();
    }
    for (int t = hl; t < L; t += 16) {
      const float2 o = s_acc[t];
      P.out[ob + t] = df_to_double({o.x, o.y});
    }
    __syncwarp();
  }
}

// ------------------------------------------------------------------- KMK --
// Square root of a positive double-float: one Newton step from the FP32 root.
__device__ __forceinline__ df df_sqrt(df x) {
  const float s0 = sqrtf(x.hi);
  const float p = s0 * s0;
  const float pe = fmaf(s0, s0, -p);
  const float res = ((x.hi - p) - pe) + x.lo;  // x - s0^2
  return df_fast_two_sum(s0, res / (2.0f * s0));
}

__device__ __forceinline__ df df_scale(df x, float c) {  // exact for c a power of two only
  return {x.hi * c, x.lo * c};
}

// Largest eigenvalue of a symmetric 3x3 double-float matrix (m00, m01, m02,
// m11, m12, m22): the trigonometric solution of the characteristic cubic in
// FP32, then one double-float Newton step on det(m - l I) = 0 (skipped when
// the step is not small, i.e. at a nearly repeated root, where the products
// below only see the eigenvalues through symmetric functions that a split
// error leaves unchanged to first order).
__device__ __forceinline__ df lmax_sym3(const df* m, df det_m) {
  const float f0 = m[0].hi, f1 = m[1].hi, f2 = m[2].hi, f3 = m[3].hi, f4 = m[4].hi, f5 = m[5].hi;
  const float q = (f0 + f3 + f5) * (1.0f / 3.0f);
  const float p1 = f1 * f1 + f2 * f2 + f4 * f4;
  const float d0 = f0 - q, d1 = f3 - q, d2 = f5 - q;
  const float p2 = d0 * d0 + d1 * d1 + d2 * d2 + 2.0f * p1;
  float l = q;
  if (p2 > 0.0f) {
    const float p = sqrtf(p2 * (1.0f / 6.0f));
    const float ip = 1.0f / p;
    const float b0 = d0 * ip, b1 = f1 * ip, b2 = f2 * ip, b3 = d1 * ip, b4 = f4 * ip, b5 = d2 * ip;
    float r = 0.5f * (b0 * (b3 * b5 - b4 * b4) - b1 * (b1 * b5 - b4 * b2) + b2 * (b1 * b4 - b3 * b2));
    r = fminf(1.0f, fmaxf(-1.0f, r));
    l = q + 2.0f * p * __cosf(acosf(r) * (1.0f / 3.0f));
  }
  const df i1 = df_add(df_add(m[0], m[3]), m[5]);
  const df i2 = df_add(df_add(df_mul_sub_mul(m[0], m[3], m[1], m[1]), df_mul_sub_mul(m[0], m[5], m[2], m[2])),
                       df_mul_sub_mul(m[3], m[5], m[4], m[4]));
  const df x = {l, 0.0f};
  const df f = df_sub(df_mul(df_add(df_mul(df_sub(x, i1), x), i2), x), det_m);
  const df fp = df_add(df_mul(df_sub(df_mul(x, {3.0f, 0.0f}), df_scale(i1, 2.0f)), x), i2);
  if (fp.hi != 0.0f) {
    const df st = df_mul(f, df_rcp(fp));
    if (fabsf(st.hi) < 1e-4f * fabsf(l)) return df_sub(x, st);
  }
  return x;
}

struct KmkArgs {
  int32_t E;
  const int32_t* xnd;
  const double* X;
  float4* rec;  // P1 double-float row-slice records (2 float4 per slice)
};

// h_bar = edge_length_from_eigenvalue_metric(simplex_tensor(ele)) is
// m^(-1/2) for the element metric m.  Every edge e_ab satisfies
// e_ab^T m e_ab = 1 for m = 1/2 sum_b g_b g_b^T (g_b the barycentric
// gradients, sum g_b = 0, g_c . e_ab = delta_cb - delta_ca), the unique
// solution of simplex_tensor's system, so W = m^-1 = 2 J J^T - 1/2 (J 1)(J 1)^T
// (Sherman-Morrison on I + 1 1^T) with J the edge matrix, det W = 2 det(J)^2.
// h_bar = W^(1/2) = (-W^2 + (i1^2 - i2) W + i1 i3 I) / (i1 i2 - i3) from the
// invariants of the square roots of W's eigenvalues (Cayley-Hamilton); the
// largest eigenvalue comes from W, the smallest as 1/lambda_max(m), the middle
// one from det W, so none is a small difference of large ones.  The element
// matrix 0.5 V g_a^T h_bar g_b is a stiffness matrix (its rows sum to zero),
// written as the double-float row slices {K_a0, K_a1 | K_a2, 0} of the P1
// assembly, all in double-float on the FP32 pipes.
__global__ void __launch_bounds__(256) k_kmk_elem(KmkArgs A) {
  note_launch();
  extern __shared__ float4 kstage_all[];
  const int lane = threadIdx.x & 31;
  float4* stage = kstage_all + (threadIdx.x >> 5) * (32 * 9);  // padded records
  for (int base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < A.E; base += gridDim.x * blockDim.x) {
    const int e = base + lane;
    if (e < A.E) {
      const int4 v = __ldg(reinterpret_cast<const int4*>(A.xnd) + e);
      const int vi[4] = {v.x, v.y, v.z, v.w};
      double x[4][3];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int a = 0; a < 3; ++a) x[i][a] = __ldg(A.X + (uint32_t)(3 * vi[i] + a));
      df J[3][3];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) J[a][b] = df_from_double(x[b][a] - x[3][a]);
      df c[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, k1 = (k + 1) % 3, k2 = (k + 2) % 3;
          c[i][k] = df_mul_sub_mul(J[i1][k1], J[i2][k2], J[i2][k1], J[i1][k2]);
        }
      const df det = df_dot3(J[0][0], c[0][0], J[1][0], c[1][0], J[2][0], c[2][0]);
      // g_b * det = column b of c; the fourth is minus their sum
      df g[4][3];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        g[0][a] = c[a][0];
        g[1][a] = c[a][1];
        g[2][a] = c[a][2];
        g[3][a] = df_neg(df_add(df_add(c[a][0], c[a][1]), c[a][2]));
      }
      df j1[3];
#pragma unroll
      for (int a = 0; a < 3; ++a) j1[a] = df_add(df_add(J[a][0], J[a][1]), J[a][2]);
      const df det2 = df_mul(det, det);
      const df im = df_scale(df_rcp(det2), 0.5f);
      df W[6], M[6];
      const int ix[6][2] = {{0, 0}, {0, 1}, {0, 2}, {1, 1}, {1, 2}, {2, 2}};
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const int r = ix[k][0], q = ix[k][1];
        W[k] = df_sub(df_scale(df_dot3(J[r][0], J[q][0], J[r][1], J[q][1], J[r][2], J[q][2]), 2.0f),
                      df_scale(df_mul(j1[r], j1[q]), 0.5f));
        M[k] = df_mul(im, df_add(df_dot3(g[0][r], g[0][q], g[1][r], g[1][q], g[2][r], g[2][q]),
                                 df_mul(g[3][r], g[3][q])));
      }
      const df dW = df_scale(det2, 2.0f);  // det W; det m = 1 / det W
      const df l1 = lmax_sym3(W, dW);
      const df l3 = df_rcp(lmax_sym3(M, df_rcp(dW)));
      const df l2 = df_mul(dW, df_rcp(df_mul(l1, l3)));
      const df s1 = df_sqrt(l1), s2 = df_sqrt(l2), s3 = df_sqrt(l3);
      const df i1 = df_add(df_add(s1, s2), s3);
      const df i2 = df_add(df_add(df_mul(s1, s2), df_mul(s2, s3)), df_mul(s1, s3));
      const df i3 = df_mul(df_mul(s1, s2), s3);
      const df cw = df_sub(df_mul(i1, i1), i2), ci = df_mul(i1, i3);
      const df den = df_rcp(df_sub(df_mul(i1, i2), i3));
      // H = W^(1/2) (symmetric): (-W^2 + cw W + ci I) den
      const df Wf[3][3] = {{W[0], W[1], W[2]}, {W[1], W[3], W[4]}, {W[2], W[4], W[5]}};
      df H[3][3];
#pragma unroll
      for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int q = r; q < 3; ++q) {
          const df w2 = df_dot3(Wf[r][0], Wf[0][q], Wf[r][1], Wf[1][q], Wf[r][2], Wf[2][q]);
          df h = df_sub(df_mul(cw, Wf[r][q]), w2);
          if (r == q) h = df_add(h, ci);
          H[r][q] = df_mul(h, den);
          H[q][r] = H[r][q];
        }
      // 0.5 * V * g_a^T H g_b with g = c / det, V = |det| / 6
      const df ks = df_rcp(df_mul(df_abs(det), {12.0f, 0.0f}));
      df hg[4][3];
#pragma unroll
      for (int b = 0; b < 4; ++b)
#pragma unroll
        for (int r = 0; r < 3; ++r) hg[b][r] = df_dot3(H[r][0], g[b][0], H[r][1], g[b][1], H[r][2], g[b][2]);
      df K[4][3];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = a; b < 3; ++b) {
          K[a][b] = df_mul(ks, df_dot3(g[a][0], hg[b][0], g[a][1], hg[b][1], g[a][2], hg[b][2]));
          K[b][a] = K[a][b];
        }
      // row 3 as the row pass rebuilds column 3 (an exactly symmetric matrix)
#pragma unroll
      for (int b = 0; b < 3; ++b) K[3][b] = df_neg(df_add(df_add(K[b][0], K[b][1]), K[b][2]));
      float4* rec = stage + lane * 9;
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        rec[2 * i] = make_float4(K[i][0].hi, K[i][0].lo, K[i][1].hi, K[i][1].lo);
        rec[2 * i + 1] = make_float4(K[i][2].hi, K[i][2].lo, 0.0f, 0.0f);
      }
    }
    __syncwarp();
    float4* out = A.rec + (uint32_t)base * 8u;
    const int nvalid = min(32, A.E - base) * 8;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int idx = k * 32 + lane;
      if (idx < nvalid) out[idx] = stage[stage_pos<8>(k, lane)];
    }
    __syncwarp();
  }
}

// ------------------------------------------------------ projection vectors --
__global__ void k_poisson_rhs(int32_t N, const int32_t* __restrict__ findrm, const int32_t* __restrict__ colm,
                              const double* __restrict__ c0, const double* __restrict__ c1,
                              const double* __restrict__ c2, const double* __restrict__ mom,
                              const double* __restrict__ ct_rhs, const double* __restrict__ iml,
                              const double* __restrict__ u, double s, double* __restrict__ out) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x) {
    double y = 0.0;
    for (int p = findrm[i]; p < findrm[i + 1]; ++p) {
      const int k = colm[p];
      const double l0 = (mom ? mom[3 * k] * iml[3 * k] : 0.0) + u[3 * k] * s;
      const double l1 = (mom ? mom[3 * k + 1] * iml[3 * k + 1] : 0.0) + u[3 * k + 1] * s;
      const double l2 = (mom ? mom[3 * k + 2] * iml[3 * k + 2] : 0.0) + u[3 * k + 2] * s;
      y += c0[p] * l0 + c1[p] * l1 + c2[p] * l2;
    }
    out[i] = -y + (ct_rhs ? ct_rhs[i] * s : 0.0);
  }
}

__global__ void k_correct_velocity(int32_t N, const int32_t* __restrict__ findrm, const int32_t* __restrict__ colm,
                                   const int32_t* __restrict__ tpos, const double* __restrict__ c0,
                                   const double* __restrict__ c1, const double* __restrict__ c2,
                                   const double* __restrict__ iml, const double* __restrict__ dp,
                                   double* __restrict__ u) {
  note_launch();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < N; k += gridDim.x * blockDim.x) {
    double d0 = 0.0, d1 = 0.0, d2 = 0.0;
    for (int r = findrm[k]; r < findrm[k + 1]; ++r) {
      const int i = colm[r], t = tpos[r];
      const double x = dp[i];
      d0 += c0[t] * x;
      d1 += c1[t] * x;
      d2 += c2[t] * x;
    }
    u[3 * k] += d0 * iml[3 * k];
    u[3 * k + 1] += d1 * iml[3 * k + 1];
    u[3 * k + 2] += d2 * iml[3 * k + 2];
  }
}

__global__ void k_axpy(int64_t n, double a, const double* __restrict__ x, double* __restrict__ y) {
  note_launch();
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x)
    y[k] += a * x[k];
}

// ----------------------------------------------------------- host helpers --
int ensure_tpos(fl_mesh_t* m, cudaStream_t s) {
  if (m->tpos.p) return FL_OK;
  FL_TRY(m->tpos.reserve((size_t)m->nnz));
  k_tpos<<<grid_for(m->N, kT), kT, 0, s>>>(m->N, m->findrm.p, m->colm.p, m->tpos.p, m->err.p);
  FL_TRY_CUDA(cudaGetLastError());
  const int st = check_err(m->err.p, s, "the pattern is not structurally symmetric");
  if (st != FL_OK) m->tpos.release();
  return st;
}

bool p1_mesh(const fl_mesh_t* m) { return m && m->E > 0 && m->loc == 4; }

template <int THREADS, int RMAX, bool CT, bool BP>
int launch_div_rows(const DivRowArgs& R, cudaStream_t s) {
  const size_t smem = CT ? (size_t)3 * RMAX * THREADS * sizeof(float2) : 0;
  static bool configured = false;
  if (!configured && smem > 48 * 1024) {
    FL_TRY_CUDA(cudaFuncSetAttribute(k_div_rows<THREADS, RMAX, CT, BP>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured = true;
  }
  const unsigned grid = (unsigned)((R.N + THREADS - 1) / THREADS);
  k_div_rows<THREADS, RMAX, CT, BP><<<grid, THREADS, smem, s>>>(R);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

// Element and row passes: CT blocks (when ct0 is given) and lumped masses.
int divergence_passes(fl_mesh_t* m, bool by_parts, double* ct0, double* ct1, double* ct2, double* ct_rhs,
                      double* dml, double* gml, cudaStream_t s) {
  FL_TRY(m->em.reserve((size_t)m->E * 10));  // 80 B per element
  DivElemArgs A{m->E, m->xndglno.p, m->coords.p, reinterpret_cast<float4*>(m->em.p), df_host(1.0 / 24.0)};
  const unsigned g = grid_for(m->E, 256, 16);
  k_div_elem<<<g, 256, (256 / 32) * 160 * sizeof(float4), s>>>(A);
  FL_TRY_CUDA(cudaGetLastError());
  DivRowArgs R{m->N, m->ne_ptr.p, m->ne_col.p, m->ne_pos.p, m->findrm.p, reinterpret_cast<const float4*>(m->em.p),
               ct0, ct1, ct2, ct_rhs, dml, gml};
  if (!ct0) return launch_div_rows<128, 16, false, false>(R, s);
  if (m->max_row <= 16)
    return by_parts ? launch_div_rows<128, 16, true, true>(R, s) : launch_div_rows<128, 16, true, false>(R, s);
  return by_parts ? launch_div_rows<64, 32, true, true>(R, s) : launch_div_rows<64, 32, true, false>(R, s);
}

// ------------------------------------------- Taylor-Hood divergence (P2/P1) --
// assemble_divergence_matrix_cg (Divergence_Matrix_CG.F90:67-375) for P1
// pressure on the vertices and P2 velocity, the element terms: with the
// divergence element records (sign(det) cof / 24 per element, double-float),
//   not by parts: C_d(a, j) = int N_a dN_j/dx_d = sum_c 24 T(a, j, c) rec(d, c),
//                 T(a, j, c) = sum_g w_g N_a(g) dN_j/dL_c(g)
//   by parts:     C_d(a, j) = -int dN_a/dx_d N_j = -sum_c 24 Tb(a, j, c) rec(d, c),
//                 Tb(a, j, c) = sum_g w_g dN_a/dL_c(g) N_j(g)
// (dN/dx_d = sum_c dN/dL_c cof(d, c) / det).  One warp per pressure row adds
// its elements in ascending element order (the reference's element loop
// order); lanes (d, j) of an element write distinct slots of the row's
// double-float accumulators in shared memory.
struct ThTensor {
  float2 t[4][10][3];  // 24 T or -24 Tb, double-float
};

struct ThArgs {
  int32_t Np;
  const int32_t* vne_ptr;
  const int32_t* vne;      // vertex -> element << 4 | local vertex, element ascending
  const int32_t* nd2;      // P2 connectivity, 10 per element
  const int32_t* findrm;   // rectangular pattern
  const int32_t* colm;
  const float4* rec;       // 5 float4 per element
  double* ct0;
  double* ct1;
  double* ct2;
  ErrWord* err;
};

constexpr int kThWarps = 4;
constexpr int kThMaxRow = 192;

__global__ void __launch_bounds__(kThWarps * 32) k_div_rows_th(ThArgs A, ThTensor T) {
  note_launch();
  __shared__ int32_t cols[kThWarps][kThMaxRow];
  __shared__ float2 acc[kThWarps][3][kThMaxRow];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int j = lane % 10, d = lane / 10;  // lanes 0..29: (component, velocity node)
  for (int row = blockIdx.x * kThWarps + w; row < A.Np; row += gridDim.x * kThWarps) {
    const int base = __ldg(A.findrm + row), L = __ldg(A.findrm + row + 1) - base;
    if (L > kThMaxRow) {
      if (lane == 0) set_err(A.err, FL_ERR_UNSUPPORTED, row);
      continue;
    }
    for (int k = lane; k < L; k += 32) {
      cols[w][k] = __ldg(A.colm + base + k);
      acc[w][0][k] = acc[w][1][k] = acc[w][2][k] = make_float2(0.0f, 0.0f);
    }
    __syncwarp();
    const int ib = __ldg(A.vne_ptr + row), ie = __ldg(A.vne_ptr + row + 1);
    for (int q = ib; q < ie; ++q) {
      const int inc = __ldg(A.vne + q);
      const int e = inc >> 4, a = inc & 15;
      int pos = -1;
      if (lane < 10) {
        const int node = __ldg(A.nd2 + (int64_t)e * 10 + lane);
        int lo = 0, hi = L - 1;
        while (lo <= hi) {
          const int mid = (lo + hi) >> 1, c = cols[w][mid];
          if (c == node) {
            pos = mid;
            break;
          }
          if (c < node) lo = mid + 1;
          else hi = mid - 1;
        }
      }
      const int pj = __shfl_sync(0xffffffffu, pos, j);
      if (lane < 30) {
        const float4* r = A.rec + (uint32_t)e * 5u;
        float v[6];
        const float4 r0 = __ldg(r + (3 * d) / 2), r1 = __ldg(r + (3 * d) / 2 + 1);
        // record entries 3d..3d+2 (two per float4: hi, lo pairs)
        v[0] = r0.x; v[1] = r0.y; v[2] = r0.z; v[3] = r0.w; v[4] = r1.x; v[5] = r1.y;
        const int o = (3 * d) & 1;  // entry 3d starts in the second half of its float4 when odd
        df c[3];
        if (o == 0) {
          c[0] = {v[0], v[1]}; c[1] = {v[2], v[3]}; c[2] = {v[4], v[5]};
        } else {
          const float4 r2 = __ldg(r + (3 * d) / 2 + 1);
          c[0] = {v[2], v[3]}; c[1] = {r2.x, r2.y}; c[2] = {r2.z, r2.w};
        }
        const float2 t0 = T.t[a][j][0], t1 = T.t[a][j][1], t2 = T.t[a][j][2];
        const df val = df_dot3({t0.x, t0.y}, c[0], {t1.x, t1.y}, c[1], {t2.x, t2.y}, c[2]);
        if (pj < 0) {
          set_err(A.err, FL_ERR_OUTSIDE_PATTERN, row);
        } else {
          const float2 s0 = acc[w][d][pj];
          const df sum = df_add({s0.x, s0.y}, val);
          acc[w][d][pj] = make_float2(sum.hi, sum.lo);
        }
      }
      __syncwarp();
    }
    for (int k = lane; k < L; k += 32) {
      const float2 x0 = acc[w][0][k], x1 = acc[w][1][k], x2 = acc[w][2][k];
      A.ct0[base + k] = df_to_double({x0.x, x0.y});
      A.ct1[base + k] = df_to_double({x1.x, x1.y});
      A.ct2[base + k] = df_to_double({x2.x, x2.y});
    }
    __syncwarp();
  }
}

static int th_tensor(int quad_degree, bool by_parts, ThTensor& T) {
  TetQuad q;
  if (!tet_quadrature(quad_degree, q)) return FL_ERR_ARG;
  TetShape p1, p2;
  tet_shape(1, q, p1);
  tet_shape(2, q, p2);
  for (int a = 0; a < 4; ++a)
    for (int jj = 0; jj < 10; ++jj)
      for (int c = 0; c < 3; ++c) {
        double s = 0.0;
        for (int g = 0; g < q.ngi; ++g)
          s += q.w[g] * (by_parts ? p1.dn[a][g][c] * p2.n[jj][g] : p1.n[a][g] * p2.dn[jj][g][c]);
        const df h = df_host(by_parts ? -24.0 * s : 24.0 * s);
        T.t[a][jj][c] = make_float2(h.hi, h.lo);
      }
  return FL_OK;
}

}  // namespace
}  // namespace fl

namespace fl {
namespace {

// The product handle h of a first factor with pattern (fr, cm) (N rows, annz
// entries) and a second factor whose rows, transposed, are (tr, tc): the
// output pattern (make_sparsity_transpose, femtools/Sparsity_Patterns.F90:
// 87-148) and the slot map of the row products.
int build_product(fl_mesh_t* h, int N, const int32_t* fr, const int32_t* cm, int64_t annz, const int32_t* tr,
                  const int32_t* tc, cudaStream_t s) {
  h->N = N;
  DevBuf<int32_t> cnt, mr;
  FL_TRY(h->err.reserve(1));
  FL_TRY(cnt.reserve(N + 1));
  FL_TRY(mr.reserve(1));
  FL_TRY(h->findrm.reserve(N + 1));
  FL_TRY(h->centrm.reserve(N));
  FL_TRY_CUDA(cudaMemsetAsync(h->err.p, 0, sizeof(ErrWord), s));
  FL_TRY_CUDA(cudaMemsetAsync(mr.p, 0, sizeof(int32_t), s));
  const unsigned g = (unsigned)std::max(1, std::min((N + kSoWarps - 1) / kSoWarps, num_sms() * 16));
  k_so_rows<<<g, kSoWarps * 32, 0, s>>>(N, fr, cm, tr, tc, nullptr, cnt.p, nullptr, nullptr, mr.p, h->err.p, 0);
  FL_TRY(check_err(h->err.p, s, "second-order row with more candidates than the row scratch holds"));
  FL_TRY(exclusive_scan_i32(cnt.p, h->findrm.p, N, s));
  int32_t nnz = 0, maxrow = 0;
  FL_TRY_CUDA(cudaMemcpyAsync(&nnz, h->findrm.p + N, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaMemcpyAsync(&maxrow, mr.p, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  h->nnz = nnz;
  h->max_row = maxrow;
  FL_TRY(h->colm.reserve((size_t)std::max(nnz, 1)));
  k_fill_i32<<<grid_for(N, kT), kT, 0, s>>>(h->centrm.p, N, -1);
  k_so_rows<<<g, kSoWarps * 32, 0, s>>>(N, fr, cm, tr, tc, h->findrm.p, nullptr, h->colm.p, h->centrm.p, mr.p,
                                        h->err.p, 1);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  // slot map of the row products
  DevBuf<int32_t> pc;
  FL_TRY(pc.reserve((size_t)annz + 1));
  FL_TRY(h->pair_off.reserve((size_t)annz + 1));
  k_pair_count<<<grid_for(annz, kT), kT, 0, s>>>(N, fr, cm, tr, pc.p);
  FL_TRY(exclusive_scan_i32(pc.p, h->pair_off.p, annz, s));
  int32_t npairs = 0;
  FL_TRY_CUDA(cudaMemcpyAsync(&npairs, h->pair_off.p + annz, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  FL_TRY(h->pair_map.reserve((size_t)std::max(npairs, 1)));
  k_pair_map<<<(unsigned)std::max(1, std::min((N + 7) / 8, num_sms() * 8)), 256, 0, s>>>(
      N, fr, cm, tr, tc, h->findrm.p, h->colm.p, h->pair_off.p, h->pair_map.p, h->err.p);
  return check_err(h->err.p, s, "second-order row longer than the product's shared-memory row");
}

fl_mesh_t* new_product_handle(int* st) {
  fl_mesh_t* h = new fl_mesh_t();
  cudaGetDevice(&h->device);
  if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("cudaStreamCreate failed");
    *st = FL_ERR_CUDA;
  }
  return h;
}

// C's pattern transposed: per column k the rows holding it (ascending) and
// the position of each such entry in C.
__global__ void k_tr_count(int32_t N, const int32_t* __restrict__ fr, const int32_t* __restrict__ cm, int32_t ncol,
                           int32_t* __restrict__ cnt, ErrWord* err) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    for (int p = fr[i]; p < fr[i + 1]; ++p) {
      const int k = cm[p];
      if (k < 0 || k >= ncol) set_err(err, FL_ERR_ARG, i);
      else atomicAdd(cnt + k, 1);
    }
}

__global__ void k_tr_fill(int32_t N, const int32_t* __restrict__ fr, const int32_t* __restrict__ cm, int32_t ncol,
                          const int32_t* __restrict__ tptr, int32_t* __restrict__ fill, int32_t* __restrict__ tcol,
                          int32_t* __restrict__ tpos) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < N; i += gridDim.x * blockDim.x)
    for (int p = fr[i]; p < fr[i + 1]; ++p) {
      const int k = cm[p];
      if (k < 0 || k >= ncol) continue;
      const int slot = tptr[k] + atomicAdd(fill + k, 1);
      tcol[slot] = i;
      tpos[slot] = p;
    }
}

__global__ void k_tr_sort(int32_t ncol, const int32_t* __restrict__ tptr, int32_t* __restrict__ tcol,
                          int32_t* __restrict__ tpos) {
  note_launch();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ncol; k += gridDim.x * blockDim.x) {
    const int b = tptr[k], e = tptr[k + 1];
    for (int a = b + 1; a < e; ++a) {
      const int x = tcol[a], y = tpos[a];
      int j = a - 1;
      while (j >= b && tcol[j] > x) {
        tcol[j + 1] = tcol[j];
        tpos[j + 1] = tpos[j];
        --j;
      }
      tcol[j + 1] = x;
      tpos[j + 1] = y;
    }
  }
}

}  // namespace
}  // namespace fl

using namespace fl;

// The second-order pattern of a P1 mesh as a pattern-only handle.
extern "C" int fl_gpu_secondorder_register(fl_mesh mesh, fl_mesh* out) {
  FL_CHECK_ARG(mesh && out, "null argument");
  FL_CHECK_ARG(mesh->N > 0 && mesh->findrm.p && mesh->colm.p, "the mesh has no pattern");
  cudaStream_t s = mesh->stream;
  FL_TRY(ensure_tpos(mesh, s));
  int st = FL_OK;
  fl_mesh_t* h = new_product_handle(&st);
  if (st == FL_OK) {
    h->so_parent = mesh;
    st = build_product(h, mesh->N, mesh->findrm.p, mesh->colm.p, mesh->nnz, mesh->findrm.p, mesh->colm.p, s);
  }
  if (st != FL_OK) {
    fl_gpu_mesh_destroy(h);
    return st;
  }
  *out = h;
  return FL_OK;
}

// The product pattern C C^T of a Taylor-Hood divergence pattern (pressure
// rows, P2 velocity columns), the pattern of its cmc_m.
extern "C" int fl_gpu_rect_secondorder_register(fl_mesh pattern, fl_mesh* out) {
  FL_CHECK_ARG(pattern && out, "null argument");
  FL_CHECK_ARG(pattern->so_parent && pattern->so_parent->loc == 10 && pattern->N == pattern->so_parent->Nx,
               "a Taylor-Hood pattern (fl_gpu_rect_register)");
  const int ncol = pattern->so_parent->N;
  const int64_t annz = pattern->nnz;
  cudaStream_t s = pattern->so_parent->stream;
  int st = FL_OK;
  fl_mesh_t* h = new_product_handle(&st);
  do {
    if (st != FL_OK) break;
    h->a_pat = pattern;
    DevBuf<int32_t> cnt;
    if ((st = h->err.reserve(1)) || (st = cnt.reserve((size_t)ncol + 1)) ||
        (st = h->tr_ptr.reserve((size_t)ncol + 1)) || (st = h->tr_col.reserve((size_t)std::max<int64_t>(annz, 1))) ||
        (st = h->tr_pos.reserve((size_t)std::max<int64_t>(annz, 1))))
      break;
    if (cudaMemsetAsync(h->err.p, 0, sizeof(ErrWord), s) != cudaSuccess ||
        cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * ((size_t)ncol + 1), s) != cudaSuccess) {
      set_error("memset failed");
      st = FL_ERR_CUDA;
      break;
    }
    k_tr_count<<<grid_for(pattern->N, kT), kT, 0, s>>>(pattern->N, pattern->findrm.p, pattern->colm.p, ncol, cnt.p,
                                                      h->err.p);
    if ((st = check_err(h->err.p, s, "a pattern column outside the velocity nodes")) != FL_OK) break;
    if ((st = exclusive_scan_i32(cnt.p, h->tr_ptr.p, ncol, s)) != FL_OK) break;
    if (cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * ((size_t)ncol + 1), s) != cudaSuccess) {
      set_error("memset failed");
      st = FL_ERR_CUDA;
      break;
    }
    k_tr_fill<<<grid_for(pattern->N, kT), kT, 0, s>>>(pattern->N, pattern->findrm.p, pattern->colm.p, ncol,
                                                     h->tr_ptr.p, cnt.p, h->tr_col.p, h->tr_pos.p);
    k_tr_sort<<<grid_for(ncol, kT), kT, 0, s>>>(ncol, h->tr_ptr.p, h->tr_col.p, h->tr_pos.p);
    if (cudaGetLastError() != cudaSuccess) {
      set_error("transposed pattern failed");
      st = FL_ERR_CUDA;
      break;
    }
    st = build_product(h, pattern->N, pattern->findrm.p, pattern->colm.p, annz, h->tr_ptr.p, h->tr_col.p, s);
  } while (0);
  if (st != FL_OK) {
    fl_gpu_mesh_destroy(h);
    return st;
  }
  *out = h;
  return FL_OK;
}

namespace fl {

int node_face_lists(fl_mesh_t* m, int32_t nf, int32_t floc, const int32_t* faces, int32_t base, cudaStream_t s) {
  const int N = m->N;
  FL_TRY(m->face_cnt.reserve(N + 1));
  FL_TRY(m->face_ptr.reserve(N + 1));
  FL_TRY(m->face_list.reserve((size_t)floc * nf));
  FL_TRY_CUDA(cudaMemsetAsync(m->face_cnt.p, 0, sizeof(int32_t) * (N + 1), s));
  k_face_count<<<grid_for((int64_t)floc * nf, kT), kT, 0, s>>>(nf, floc, faces, base, N, m->face_cnt.p, m->err.p);
  FL_TRY(check_err(m->err.p, s, "surface face node out of range"));
  FL_TRY(exclusive_scan_i32(m->face_cnt.p, m->face_ptr.p, N, s));
  FL_TRY_CUDA(cudaMemsetAsync(m->face_cnt.p, 0, sizeof(int32_t) * (N + 1), s));
  k_face_fill<<<grid_for((int64_t)floc * nf, kT), kT, 0, s>>>(nf, floc, faces, base, N, m->face_ptr.p,
                                                              m->face_cnt.p, m->face_list.p);
  k_face_sort<<<grid_for(N, kT), kT, 0, s>>>(N, m->face_ptr.p, m->face_list.p);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

}  // namespace fl

extern "C" int fl_dev_assemble_divergence_cg(fl_mesh m, const fl_divergence_params* p, double* const ct_val[3],
                                             double* ct_rhs, double* div_mass_lumped, double* grad_mass_lumped,
                                             void* stream) {
  FL_CHECK_ARG(p1_mesh(m), "a P1 mesh handle (P1 pressure and velocity on one mesh)");
  FL_CHECK_ARG(p && ct_val && ct_val[0] && ct_val[1] && ct_val[2], "null argument");
  FL_CHECK_ARG(p->index_base == 0 || p->index_base == 1, "index_base");
  const bool bp = p->integrate_by_parts != 0;
  FL_CHECK_ARG(!bp || p->nfaces == 0 || (p->faces && p->face_ele), "faces and face_ele");
  cudaStream_t s = pick(m, stream);
  FL_TRY(divergence_passes(m, bp, ct_val[0], ct_val[1], ct_val[2], ct_rhs, div_mass_lumped, grad_mass_lumped, s));
  if (bp && p->nfaces > 0) {
    const int N = m->N;
    FL_TRY(node_face_lists(m, p->nfaces, 3, p->faces, p->index_base, s));
    FaceArgs F{N, p->index_base, m->face_ptr.p, m->face_list.p, p->faces, p->face_ele, p->bc_type, p->bc_val,
               m->xndglno.p, m->coords.p, m->findrm.p, m->colm.p, ct_val[0], ct_val[1], ct_val[2], ct_rhs,
               m->E, m->err.p};
    k_div_faces<<<grid_for(N, 128), 128, 0, s>>>(F);
    FL_TRY_CUDA(cudaGetLastError());
  }
  return check_err(m->err.p, s, "divergence assembly");
}

extern "C" int fl_dev_assemble_divergence_p2p1_faces(fl_mesh m, fl_mesh rect, const fl_divergence_params* p,
                                                    const int32_t* vfaces, int32_t quad_degree,
                                                    double* const ct_val[3], double* ct_rhs, void* stream) {
  FL_CHECK_ARG(m && rect && p && ct_val && ct_val[0] && ct_val[1] && ct_val[2], "null argument");
  FL_CHECK_ARG(m->loc == 10 && m->E > 0, "a P2 (velocity) mesh handle");
  FL_CHECK_ARG(rect->so_parent == m && rect->N == m->Nx, "the rectangular pattern of this mesh (fl_gpu_rect_register)");
  FL_CHECK_ARG(p->index_base == 0 || p->index_base == 1, "index_base");
  if (p->nfaces <= 0) return FL_OK;
  FL_CHECK_ARG(p->faces && p->face_ele && vfaces, "faces, face_ele and vfaces");
  ThFaceArgs A{};
  double l[6][3], w[6];
  const int ngi = tri_rule(quad_degree, l, w);
  FL_CHECK_ARG(ngi > 0, "quadrature degree 1..4");
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 6; ++j) A.T[i][j] = 0.0;
  for (int g = 0; g < ngi; ++g) {
    double Lp[3], Nu[6];
    tri_lagrange(3, l[g], Lp);
    tri_lagrange(6, l[g], Nu);
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 6; ++j) A.T[i][j] += w[g] * (Lp[i] * Nu[j]);
  }
  cudaStream_t s = pick(m, stream);
  const int N = rect->N;
  FL_TRY(node_face_lists(rect, p->nfaces, 3, p->faces, p->index_base, s));
  A.F = FaceArgs{N, p->index_base, rect->face_ptr.p, rect->face_list.p, p->faces, p->face_ele, p->bc_type,
                 p->bc_val, m->xndglno.p, m->coords.p, rect->findrm.p, rect->colm.p, ct_val[0], ct_val[1],
                 ct_val[2], ct_rhs, m->E, rect->err.p};
  A.vfaces = vfaces;
  k_div_faces_th<<<grid_for(N, 128), 128, 0, s>>>(A);
  FL_TRY_CUDA(cudaGetLastError());
  return check_err(rect->err.p, s, "Taylor-Hood divergence surface terms");
}

namespace fl {
namespace {

// compute_lumped_mass of a P2 mesh (unit density): the row sums of
// shape_shape over the rule, |detJ| sum_g w_g N_i(g) sum_j N_j(g) =
// |detJ| W_i with W_i = sum_g w_g N_i(g) (the P2 functions sum to one; the
// degree-4 rule is exact: W = -1/120 at the vertices, 1/30 at the edges).
// One thread per node over its elements in ascending order (the element
// loop's order of the reference's addto).
struct LumpP2Args {
  int32_t N;
  const int32_t* ne_ptr;
  const int32_t* ne;
  const double* adet;  // |detJ| of every element
  double W[10];
  double* out;
};

// |detJ| of every element, once (FP64: one determinant per element instead
// of one per incidence)
__global__ void k_abs_det(int32_t E, const int32_t* __restrict__ xnd, const double* __restrict__ X,
                          double* __restrict__ adet) {
  note_launch();
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
    double x[4][3];
    for (int i = 0; i < 4; ++i)
      for (int c = 0; c < 3; ++c) x[i][c] = X[3 * xnd[4 * e + i] + c];
    double J[3][3];
    for (int c = 0; c < 3; ++c)
      for (int b = 0; b < 3; ++b) J[c][b] = x[b][c] - x[3][c];
    const double det = J[0][0] * (J[1][1] * J[2][2] - J[2][1] * J[1][2]) -
                       J[1][0] * (J[0][1] * J[2][2] - J[2][1] * J[0][2]) +
                       J[2][0] * (J[0][1] * J[1][2] - J[1][1] * J[0][2]);
    adet[e] = fabs(det);
  }
}

__global__ void k_lumped_p2(LumpP2Args A) {
  note_launch();
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < A.N; v += gridDim.x * blockDim.x) {
    double sum = 0.0;
    for (int q = A.ne_ptr[v]; q < A.ne_ptr[v + 1]; ++q) {
      const int inc = A.ne[q];
      sum += A.adet[inc >> 4] * A.W[inc & 15];
    }
    A.out[v] = sum;
  }
}

}  // namespace
}  // namespace fl

extern "C" int fl_dev_lumped_mass(fl_mesh m, double* lumped_mass, void* stream) {
  FL_CHECK_ARG(m && m->E > 0 && (m->loc == 4 || m->loc == 10), "a P1 or P2 mesh handle");
  FL_CHECK_ARG(lumped_mass, "null argument");
  cudaStream_t s = pick(m, stream);
  if (m->loc == 4) {
    FL_TRY(divergence_passes(m, false, nullptr, nullptr, nullptr, nullptr, lumped_mass, nullptr, s));
    return FL_OK;
  }
  TetQuad q;
  tet_quadrature(4, q);
  TetShape sh;
  tet_shape(2, q, sh);
  FL_TRY(m->em.reserve((size_t)m->E));
  k_abs_det<<<grid_for(m->E, kT), kT, 0, s>>>(m->E, m->xndglno.p, m->coords.p, m->em.p);
  LumpP2Args A{m->N, m->ne_ptr.p, m->ne.p, m->em.p, {}, lumped_mass};
  for (int i = 0; i < 10; ++i) {
    double w = 0.0;
    for (int g = 0; g < q.ngi; ++g) w += q.w[g] * sh.n[i][g];
    A.W[i] = w;
  }
  k_lumped_p2<<<grid_for(m->N, kT), kT, 0, s>>>(A);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

static int rowprod_launch(fl_mesh prod, int ndim, bool div, const double* const a[3], const double* w,
                          const double* const b[3], double theta, int scale, double* out, cudaStream_t s) {
  // first factor's pattern, and the second factor's rows transposed (for a
  // structurally symmetric square pattern, the pattern itself)
  fl_mesh_t* par = prod->a_pat ? prod->a_pat : prod->so_parent;
  const int64_t annz = par->nnz;
  const int32_t* tpos = prod->a_pat ? prod->tr_pos.p : par->tpos.p;
  FL_TRY(prod->bt.reserve((size_t)ndim * annz));
  const unsigned gb = grid_for(annz, kT);
  if (ndim == 1) k_bt_gather<1><<<gb, kT, 0, s>>>(annz, tpos, b[0], nullptr, nullptr, prod->bt.p);
  else if (ndim == 2) k_bt_gather<2><<<gb, kT, 0, s>>>(annz, tpos, b[0], b[1], nullptr, prod->bt.p);
  else k_bt_gather<3><<<gb, kT, 0, s>>>(annz, tpos, b[0], b[1], b[2], prod->bt.p);
  RowProdArgs P{};
  P.n = prod->N;
  P.annz = annz;
  P.aptr = par->findrm.p;
  P.acol = par->colm.p;
  P.tptr = prod->a_pat ? prod->tr_ptr.p : par->findrm.p;
  P.optr = prod->findrm.p;
  P.poff = prod->pair_off.p;
  P.pmap = prod->pair_map.p;
  for (int d = 0; d < 3; ++d) P.a[d] = d < ndim ? a[d] : nullptr;
  P.bt = prod->bt.p;
  P.w = w;
  P.theta = theta;
  P.scale = scale;
  P.out = out;
  P.err = prod->err.p;
  // one resident wave: blocks per SM from the occupancy of the instance
  auto launch = [&](auto kern) -> int {
    int per_sm = 0;
    FL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPW * 32, 0));
    const unsigned g = (unsigned)std::max(1, std::min((P.n + 2 * kPW - 1) / (2 * kPW), num_sms() * std::max(1, per_sm)));
    kern<<<g, kPW * 32, 0, s>>>(P);
    return FL_OK;
  };
  if (div) FL_TRY(launch(k_rowprod<1, true>));
  else if (ndim == 1) FL_TRY(launch(k_rowprod<1, false>));
  else if (ndim == 2) FL_TRY(launch(k_rowprod<2, false>));
  else FL_TRY(launch(k_rowprod<3, false>));
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

static int check_product(fl_mesh prod) {
  FL_CHECK_ARG(prod && (prod->so_parent || prod->a_pat),
               "a second-order pattern handle (fl_gpu_secondorder_register, fl_gpu_rect_secondorder_register)");
  FL_CHECK_ARG(prod->a_pat ? prod->tr_pos.p != nullptr : prod->so_parent->tpos.p != nullptr,
               "the parent pattern has no transpose map");
  return FL_OK;
}

extern "C" int fl_dev_mult_div_vector_div_T(fl_mesh prod, int32_t ndim, const double* const a_val[3],
                                            const double* w, const double* const b_val[3], double* out,
                                            void* stream) {
  FL_TRY(check_product(prod));
  FL_CHECK_ARG(ndim >= 1 && ndim <= 3, "ndim 1..3");
  FL_CHECK_ARG(a_val && b_val && w && out, "null argument");
  for (int d = 0; d < ndim; ++d) FL_CHECK_ARG(a_val[d] && b_val[d], "null block");
  return rowprod_launch(prod, ndim, false, a_val, w, b_val, 1.0, 0, out, pick(prod, stream));
}

extern "C" int fl_dev_mult_div_invscalar_div_T(fl_mesh prod, const double* a_val, const double* s_val,
                                               const double* b_val, double* out, void* stream) {
  FL_TRY(check_product(prod));
  FL_CHECK_ARG(a_val && b_val && s_val && out, "null argument");
  const double* a[3] = {a_val, nullptr, nullptr};
  const double* b[3] = {b_val, nullptr, nullptr};
  return rowprod_launch(prod, 1, true, a, s_val, b, 1.0, 0, out, pick(prod, stream));
}

extern "C" int fl_dev_assemble_kmk(fl_mesh m, fl_mesh prod, double theta_pg, const double* p_masslump,
                                   double* kt_val, double* kmk_val, void* stream) {
  FL_CHECK_ARG(p1_mesh(m), "a P1 mesh handle");
  FL_TRY(check_product(prod));
  FL_CHECK_ARG(prod->so_parent == m, "the product pattern of this mesh");
  FL_CHECK_ARG(p_masslump && kmk_val, "null argument");
  cudaStream_t s = pick(m, stream);
  double* kt = kt_val;
  if (!kt) {
    FL_TRY(m->st_val.reserve((size_t)m->nnz));
    kt = m->st_val.p;
  }
  FL_TRY(m->em.reserve((size_t)m->E * 16));  // 128 B per element
  KmkArgs K{m->E, m->xndglno.p, m->coords.p, reinterpret_cast<float4*>(m->em.p)};
  k_kmk_elem<<<grid_for(m->E, 256, 8), 256, 8 * 32 * 9 * sizeof(float4), s>>>(K);
  FL_TRY_CUDA(cudaGetLastError());
  FL_TRY(m->st_rhs.reserve((size_t)m->N));
  FL_TRY(rows_p1_df(m, m->em.p, kt, m->st_rhs.p, s));
  // by scaling masslump with theta, kmk is divided by theta (Momentum_CG.F90:2750-2762)
  const int scale = fabs(theta_pg - 1.0) < DBL_EPSILON ? 0 : 1;
  const double* a[3] = {kt, nullptr, nullptr};
  return rowprod_launch(prod, 1, true, a, p_masslump, a, theta_pg, scale, kmk_val, s);
}

extern "C" int fl_dev_masslumped_poisson_rhs(fl_mesh m, const double* const ctp_val[3], const double* mom_rhs,
                                             const double* ct_rhs, const double* inverse_masslump,
                                             const double* velocity, double dt, double theta_pg,
                                             double* poisson_rhs, void* stream) {
  FL_CHECK_ARG(m && m->N > 0 && m->findrm.p, "mesh");
  FL_CHECK_ARG(ctp_val && ctp_val[0] && ctp_val[1] && ctp_val[2] && velocity && poisson_rhs, "null argument");
  FL_CHECK_ARG(!mom_rhs || inverse_masslump, "mom_rhs needs inverse_masslump");
  FL_CHECK_ARG(dt != 0.0 && theta_pg != 0.0, "dt and theta_pg nonzero");
  cudaStream_t s = pick(m, stream);
  k_poisson_rhs<<<grid_for(m->N, kT), kT, 0, s>>>(m->N, m->findrm.p, m->colm.p, ctp_val[0], ctp_val[1], ctp_val[2],
                                                   mom_rhs, ct_rhs, inverse_masslump, velocity, 1.0 / dt / theta_pg,
                                                   poisson_rhs);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

extern "C" int fl_dev_correct_masslumped_velocity(fl_mesh m, const double* const ct_val[3],
                                                  const double* inverse_masslump, const double* delta_p,
                                                  double* velocity, void* stream) {
  FL_CHECK_ARG(m && m->N > 0 && m->findrm.p, "mesh");
  FL_CHECK_ARG(ct_val && ct_val[0] && ct_val[1] && ct_val[2] && inverse_masslump && delta_p && velocity,
               "null argument");
  cudaStream_t s = pick(m, stream);
  FL_TRY(ensure_tpos(m, s));
  k_correct_velocity<<<grid_for(m->N, kT), kT, 0, s>>>(m->N, m->findrm.p, m->colm.p, m->tpos.p, ct_val[0],
                                                        ct_val[1], ct_val[2], inverse_masslump, delta_p, velocity);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

extern "C" int fl_dev_csr_addto(fl_mesh pattern, double* val, const double* other, double scale, void* stream) {
  FL_CHECK_ARG(pattern && pattern->nnz > 0 && val && other, "null argument");
  cudaStream_t s = pick(pattern, stream);
  k_axpy<<<grid_for(pattern->nnz, kT), kT, 0, s>>>(pattern->nnz, scale, other, val);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

extern "C" int fl_dev_assemble_divergence_p2p1(fl_mesh m, fl_mesh rect, int32_t integrate_by_parts,
                                              int32_t quad_degree, double* const ct_val[3], void* stream) {
  FL_CHECK_ARG(m && rect && ct_val && ct_val[0] && ct_val[1] && ct_val[2], "null argument");
  FL_CHECK_ARG(m->loc == 10 && m->E > 0, "a P2 (velocity) mesh handle");
  FL_CHECK_ARG(rect->so_parent == m && rect->N == m->Nx, "the rectangular pattern of this mesh (fl_gpu_rect_register)");
  FL_CHECK_ARG(quad_degree >= 1 && quad_degree <= 4, "quadrature degree 1..4");
  cudaStream_t s = pick(m, stream);
  ThTensor T;
  FL_TRY(th_tensor(quad_degree, integrate_by_parts != 0, T));
  FL_TRY(m->em.reserve((size_t)m->E * 10));  // 80 B per element
  DivElemArgs D{m->E, m->xndglno.p, m->coords.p, reinterpret_cast<float4*>(m->em.p), df_host(1.0 / 24.0)};
  k_div_elem<<<grid_for(m->E, 256, 16), 256, (256 / 32) * 160 * sizeof(float4), s>>>(D);
  FL_TRY_CUDA(cudaGetLastError());
  ThArgs A{rect->N, m->vne_ptr.p, m->vne.p, m->ndglno.p, rect->findrm.p, rect->colm.p,
           reinterpret_cast<const float4*>(m->em.p), ct_val[0], ct_val[1], ct_val[2], m->err.p};
  k_div_rows_th<<<grid_for(rect->N, kThWarps * 32, 8), kThWarps * 32, 0, s>>>(A, T);
  FL_TRY_CUDA(cudaGetLastError());
  return check_err(m->err.p, s, "Taylor-Hood divergence: a row longer than the kernel's row scratch, or a "
                                "velocity node outside the pattern");
}
