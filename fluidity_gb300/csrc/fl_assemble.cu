// fl_assemble.cu -- CG advection-diffusion / Poisson element assembly into the
// device csr_matrix, and strong Dirichlet conditions.
//
// The element loop replaces the coloured OpenMP region of
// assemble_advection_diffusion_cg (assemble/Advection_Diffusion_CG.F90:560-598)
// in two passes:
//  1. an element pass computes every element's matrix and right-hand side once
//     (coalesced, one thread per element) into a coefficient-major scratch
//     buffer;
//  2. a row pass gives each CSR row to one thread, which adds the
//     contributions of the row's elements in the order of their colour in the
//     COLOURING_CG1 colouring -- the order in which the reference's coloured
//     loop adds them -- and writes the row once.
// No atomics; every entry is summed in the reference's (colour, element)
// order, so results are deterministic.
//
// Element matrices follow the term routines of Advection_Diffusion_CG.F90
// (:867 mass, :943 advection not by parts, :1143 absorption, :1164
// diffusivity, :1129 source) with the quadrature sums regrouped: every
// integral is a contraction of per-element geometric factors (|detJ|, invJ,
// nodal coefficients) with reference-element tensors that hold the
// quadrature sums over the same rule (femtools/Quadrature.F90:649-735) and the
// same Lagrange basis (femtools/Shape_Functions.F90:128-329).  The regrouping
// is exact in real arithmetic; results agree with the reference loops to
// rounding.
#include <climits>
#include <cmath>
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

#include "fl_internal.cuh"
#include "fl_device.cuh"
#include "fl_refelem.h"
#include "fl_df64.cuh"

namespace fl {

unsigned long long launches_assemble() { return unit_launches(); }

// Reference tensors for one (field degree, quadrature degree) pair; velocity
// and absorption coefficients are nodal on P1 (velocity) / the field mesh.
struct RefTensors {
  int loc, ngi;
  double wsum;
  double M[10][10];              // sum_g w N_i N_j
  double R[10][10][3][3];        // sum_g w dN_i/dL_a dN_j/dL_b
  double T[10][10][4][3];        // sum_g w N_i Nu_k dN_j/dL_a       (advection)
  double D[10][10][4][3];        // sum_g w N_i N_j dNu_k/dL_a       (beta div u)
  double W[10][10][10];          // sum_g w N_i N_j N_k              (absorption)
};

static void build_tensors(int degree, int qdeg, RefTensors& t) {
  TetQuad q;
  tet_quadrature(qdeg, q);
  TetShape s, u;
  tet_shape(degree, q, s);
  tet_shape(1, q, u);
  std::memset(&t, 0, sizeof(t));
  t.loc = s.loc;
  t.ngi = q.ngi;
  for (int g = 0; g < q.ngi; ++g) t.wsum += q.w[g];
  for (int i = 0; i < s.loc; ++i)
    for (int j = 0; j < s.loc; ++j)
      for (int g = 0; g < q.ngi; ++g) {
        const double w = q.w[g];
        t.M[i][j] += w * s.n[i][g] * s.n[j][g];
        for (int a = 0; a < 3; ++a)
          for (int b = 0; b < 3; ++b) t.R[i][j][a][b] += w * s.dn[i][g][a] * s.dn[j][g][b];
        for (int k = 0; k < 4; ++k)
          for (int a = 0; a < 3; ++a) {
            t.T[i][j][k][a] += w * s.n[i][g] * u.n[k][g] * s.dn[j][g][a];
            t.D[i][j][k][a] += w * s.n[i][g] * s.n[j][g] * u.dn[k][g][a];
          }
        for (int k = 0; k < s.loc; ++k) t.W[i][j][k] += w * s.n[i][g] * s.n[j][g] * s.n[k][g];
      }
}

// Geometry of a linear simplex element, as construct_cache computes it
// (femtools/Transform_elements.F90:258-301): J_T(a,b) = x_b - x_4 (columns of
// dn are unit vectors and -1 for the dependent coordinate), invJ by cofactors
// over cyc3, detJ = J_T(:,1).invJ(:,1).  Returns the unscaled cofactors and
// detJ; invJ = cof / detJ.
struct Geo {
  double cof[3][3];
  double det;
};

__device__ __forceinline__ void element_geo(const double* __restrict__ X, const int32_t* __restrict__ xnd,
                                            int64_t e, Geo& g) {
  const int4 v = __ldg(reinterpret_cast<const int4*>(xnd) + e);
  const int vi[4] = {v.x, v.y, v.z, v.w};
  double x[4][3];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int a = 0; a < 3; ++a) x[i][a] = __ldg(X + 3 * (int64_t)vi[i] + a);
  double J[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) J[a][b] = x[b][a] - x[3][a];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, k1 = (k + 1) % 3, k2 = (k + 2) % 3;
      g.cof[i][k] = J[i1][k1] * J[i2][k2] - J[i2][k1] * J[i1][k2];
    }
  g.det = J[0][0] * g.cof[0][0] + J[1][0] * g.cof[1][0] + J[2][0] * g.cof[2][0];
}

struct AsmArgs {
  int32_t E;
  const int32_t* nd;        // field connectivity
  const int32_t* xnd;       // coordinate connectivity (int4 per element)
  const double* X;
  const double* t;
  const double* u;
  const double* f;
  const double* alpha;
  double* em;               // element matrices: em[k * E + e]
  const RefTensors* ref;
  double theta_dt;
  double beta;
  double kappa[9];
  int have_mass, lump, have_adv, have_beta, have_diff, iso, have_src, have_abs, use_dt;
  int by_parts;             // integrate_advection_by_parts
};

// General element kernel: any term combination, P1 or P2 fields, P1
// coordinates and velocity.  One thread per element; writes the full LOC x LOC
// matrix (row-major, coefficient k = i*LOC + j) and the LOC rhs entries
// (k = LOC*LOC + i).
template <int LOC>
__global__ void __launch_bounds__(128) k_asm_general(AsmArgs A) {
  note_launch();
  const RefTensors& R = *A.ref;
  const int64_t E = A.E;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.E; e += gridDim.x * blockDim.x) {
    Geo g;
    element_geo(A.X, A.xnd, e, g);
    const double rdet = 1.0 / g.det;
    const double adet = fabs(g.det);
    double invJ[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) invJ[a][b] = g.cof[a][b] * rdet;
    int tn[LOC];
#pragma unroll
    for (int i = 0; i < LOC; ++i) tn[i] = __ldg(A.nd + (int64_t)e * LOC + i);
    double Te[LOC];
#pragma unroll
    for (int i = 0; i < LOC; ++i) Te[i] = A.t ? __ldg(A.t + tn[i]) : 0.0;
    // Diffusion factor Q(a,b) = |det| sum_cd invJ(c,a) kappa(c,d) invJ(d,b):
    // dshape_dot_dshape / dshape_tensor_dshape (FETools.F90:391,668) with
    // dshape = dn . invJ^T.
    double Q[3][3];
    if (A.have_diff) {
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) {
          double s = 0.0;
          if (A.iso) {
#pragma unroll
            for (int c = 0; c < 3; ++c) s += invJ[c][a] * invJ[c][b];
            s *= A.kappa[0];
          } else {
#pragma unroll
            for (int c = 0; c < 3; ++c)
#pragma unroll
              for (int d = 0; d < 3; ++d) s += invJ[c][a] * A.kappa[3 * c + d] * invJ[d][b];
          }
          Q[a][b] = s * adet;
        }
    }
    // Advection factor V(k,a) = |det| u_k . invJ(:,a): u at quadrature points
    // is the nodal P1 interpolant (ele_val_at_quad, Fields_Base.F90:2256).
    double V[4][3];
    if (A.have_adv) {
      const int4 v = __ldg(reinterpret_cast<const int4*>(A.xnd) + e);
      const int vi[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        double uk[3];
#pragma unroll
        for (int c = 0; c < 3; ++c) uk[c] = __ldg(A.u + 3 * (int64_t)vi[k] + c);
#pragma unroll
        for (int a = 0; a < 3; ++a) V[k][a] = (uk[0] * invJ[0][a] + uk[1] * invJ[1][a] + uk[2] * invJ[2][a]) * adet;
      }
    }
    double al[LOC];
    if (A.have_abs) {
#pragma unroll
      for (int k = 0; k < LOC; ++k) al[k] = __ldg(A.alpha + tn[k]) * adet;
    }
    double fe[LOC];
    if (A.have_src) {
#pragma unroll
      for (int k = 0; k < LOC; ++k) fe[k] = __ldg(A.f + tn[k]) * adet;
    }
#pragma unroll 1
    for (int i = 0; i < LOC; ++i) {
      double m[LOC];     // matrix row
      double op[LOC];    // operator row (advection + absorption + diffusion)
      double r = 0.0;
#pragma unroll
      for (int j = 0; j < LOC; ++j) {
        m[j] = 0.0;
        op[j] = 0.0;
      }
      if (A.have_mass) {
        if (A.lump) {
          double s = 0.0;
#pragma unroll
          for (int j = 0; j < LOC; ++j) s += R.M[i][j] * adet;
#pragma unroll
          for (int j = 0; j < LOC; ++j) m[j] = (j == i) ? s : 0.0;
        } else {
#pragma unroll
          for (int j = 0; j < LOC; ++j) m[j] = R.M[i][j] * adet;
        }
      }
      if (A.have_adv) {
        // not by parts: N_i u.grad N_j (T[i][j]) + beta N_i N_j div u;
        // by parts (:1019-1057): -(grad N_i . u) N_j (T[j][i]) - (1 - beta) N_i N_j div u
#pragma unroll
        for (int j = 0; j < LOC; ++j) {
          double s = 0.0;
#pragma unroll
          for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int a = 0; a < 3; ++a) s += V[k][a] * (A.by_parts ? R.T[j][i][k][a] : R.T[i][j][k][a]);
          if (A.by_parts) s = -s;
          if (A.have_beta) {
            double d = 0.0;
#pragma unroll
            for (int k = 0; k < 4; ++k)
#pragma unroll
              for (int a = 0; a < 3; ++a) d += V[k][a] * R.D[i][j][k][a];
            s = s + A.beta * d;
          }
          op[j] += s;
        }
      }
      if (A.have_abs) {
#pragma unroll
        for (int j = 0; j < LOC; ++j) {
          double s = 0.0;
#pragma unroll
          for (int k = 0; k < LOC; ++k) s += al[k] * R.W[i][j][k];
          op[j] += s;
        }
      }
      if (A.have_diff) {
#pragma unroll
        for (int j = 0; j < LOC; ++j) {
          double s = 0.0;
#pragma unroll
          for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b) s += Q[a][b] * R.R[i][j][a][b];
          op[j] += s;
        }
      }
#pragma unroll
      for (int j = 0; j < LOC; ++j) {
        if (A.use_dt) m[j] += A.theta_dt * op[j];
        r -= op[j] * Te[j];
      }
      if (A.have_src) {
#pragma unroll
        for (int j = 0; j < LOC; ++j) r += R.M[i][j] * fe[j];
      }
#pragma unroll
      for (int j = 0; j < LOC; ++j) A.em[(int64_t)(i * LOC + j) * E + e] = m[j];
      A.em[(int64_t)(LOC * LOC + i) * E + e] = r;
    }
  }
}

// P1 advection-diffusion element matrices in closed form, in double-float on
// the FP32 pipes: k_asm_general<4> spends ~520 FP64 operations per element,
// and GB300 runs FP64 FMAs at ~1/70 of its FP32 rate.  With P1 coordinates
// and a P1 velocity every reference tensor of the general kernel factors
// through the reference mass (m0 on the diagonal, m1 off it: the tet rules
// are symmetric under vertex permutations) and the constant reference
// gradients dn_j, exactly: T[i][j][k][a] = M[i][k] dn_j[a], D[i][j][k][a] =
// M[i][j] dn_k[a], R[i][j][a][b] = wsum dn_i[a] dn_j[b].  With c_j the
// cofactor columns (invJ dn_j = c_j / det, c_3 = -(c_0 + c_1 + c_2)),
// s = sign(det) and uc[k][j] = u_k . c_j:
//   advection   A_ij = s (m1 S_j + (m0 - m1) uc[i][j]),  S_j = sum_k uc[k][j]
//   by parts    A_ij = -s (m1 S_i + (m0 - m1) uc[j][i])
//   divergence  beta s M_ij sum_k uc[k][k]   (beta = -(1 - beta) by parts)
//   diffusion   K_ij = wsum (c_i . kappa c_j) / |det|   (diagonal kappa)
//   mass        |det| M_ij, or |det| (m0 + 3 m1) on the diagonal (lumped)
// and, as in k_asm_general<4>, the matrix M + theta dt op and the rhs
// -op T + |det| M f, written in the same em layout (k = 4 i + j, 16 + i).
struct AdvDfArgs {
  int32_t E;
  const int32_t* nd;   // field connectivity (int4 per element)
  const int32_t* xnd;  // coordinate connectivity (int4 per element)
  const double* X;
  const double* t;
  const double* u;
  const double* f;
  double* em;
  df m0, m1, dm, ml;   // reference mass: diagonal, off-diagonal, m0 - m1, m0 + 3 m1
  df kd[3];            // wsum * kappa_aa
  df qs;               // theta * dt (zero without the time term)
  df beta;             // divergence coefficient
  int have_mass, lump, by_parts, have_beta, have_diff, have_src;
};

template <bool ADV>
__global__ void __launch_bounds__(128) k_asm_p1_advdif_df(AdvDfArgs A) {
  note_launch();
  const int64_t E = A.E;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.E; e += gridDim.x * blockDim.x) {
    const int4 v = __ldg(reinterpret_cast<const int4*>(A.xnd) + e);
    const int vi[4] = {v.x, v.y, v.z, v.w};
    df c[4][3];
    df det;
    {
      double x[4][3];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int a = 0; a < 3; ++a) x[i][a] = __ldg(A.X + 3 * (int64_t)vi[i] + a);
      df J[3][3];
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
        for (int b = 0; b < 3; ++b) J[a][b] = df_from_double(x[b][a] - x[3][a]);
      df cof[3][3];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, k1 = (k + 1) % 3, k2 = (k + 2) % 3;
          cof[i][k] = df_mul_sub_mul(J[i1][k1], J[i2][k2], J[i2][k1], J[i1][k2]);
        }
      det = df_dot3(J[0][0], cof[0][0], J[1][0], cof[1][0], J[2][0], cof[2][0]);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
#pragma unroll
        for (int i = 0; i < 3; ++i) c[i][a] = cof[a][i];
        c[3][a] = df_neg(df_add(df_add(c[0][a], c[1][a]), c[2][a]));
      }
    }
    const bool neg = det.hi < 0.0f;
    const df adet = df_abs(det);
    df op[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) op[i][j] = {0.0f, 0.0f};
    if (A.have_diff) {
      const df rdet = df_rcp(adet);
      df kc[3][3];
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int a = 0; a < 3; ++a) kc[j][a] = df_mul(A.kd[a], c[j][a]);
      df G[4][4];
#pragma unroll
      for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = i; j < 3; ++j) {
          G[i][j] = df_dot3(c[i][0], kc[j][0], c[i][1], kc[j][1], c[i][2], kc[j][2]);
          G[j][i] = G[i][j];
        }
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        G[i][3] = df_neg(df_add(df_add(G[i][0], G[i][1]), G[i][2]));
        G[3][i] = G[i][3];
      }
      G[3][3] = df_neg(df_add(df_add(G[0][3], G[1][3]), G[2][3]));
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) op[i][j] = df_mul(G[i][j], rdet);
    }
    if (ADV) {
      df uc[4][4];
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        df uk[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) uk[a] = df_from_double(__ldg(A.u + 3 * (int64_t)vi[k] + a));
#pragma unroll
        for (int j = 0; j < 4; ++j) uc[k][j] = df_dot3(uk[0], c[j][0], uk[1], c[j][1], uk[2], c[j][2]);
      }
      df S[4];
#pragma unroll
      for (int j = 0; j < 4; ++j) S[j] = df_add(df_add(uc[0][j], uc[1][j]), df_add(uc[2][j], uc[3][j]));
      const bool flip = neg != (A.by_parts != 0);
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          df a = A.by_parts ? df_add(df_mul(A.m1, S[i]), df_mul(A.dm, uc[j][i]))
                            : df_add(df_mul(A.m1, S[j]), df_mul(A.dm, uc[i][j]));
          if (flip) a = df_neg(a);
          op[i][j] = df_add(op[i][j], a);
        }
      if (A.have_beta) {
        df dv = df_add(df_add(uc[0][0], uc[1][1]), df_add(uc[2][2], uc[3][3]));
        if (neg) dv = df_neg(dv);
        const df bd = df_mul(A.beta, dv);
        const df b0 = df_mul(bd, A.m0), b1 = df_mul(bd, A.m1);
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 4; ++j) op[i][j] = df_add(op[i][j], i == j ? b0 : b1);
      }
    }
    const int4 tv = __ldg(reinterpret_cast<const int4*>(A.nd) + e);
    const int tn[4] = {tv.x, tv.y, tv.z, tv.w};
    df T[4], fa[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      T[j] = A.t ? df_from_double(__ldg(A.t + tn[j])) : df{0.0f, 0.0f};
      fa[j] = A.have_src ? df_mul(adet, df_from_double(__ldg(A.f + tn[j]))) : df{0.0f, 0.0f};
    }
    const df fs = df_add(df_add(fa[0], fa[1]), df_add(fa[2], fa[3]));
    const df md = df_mul(adet, A.lump ? A.ml : A.m0), mo = df_mul(adet, A.m1);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      df r = {0.0f, 0.0f};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        df m = A.have_mass ? (i == j ? md : (A.lump ? df{0.0f, 0.0f} : mo)) : df{0.0f, 0.0f};
        m = df_add(m, df_mul(A.qs, op[i][j]));
        A.em[(int64_t)(4 * i + j) * E + e] = df_to_double(m);
        r = df_sub(r, df_mul(op[i][j], T[j]));
      }
      if (A.have_src) r = df_add(r, df_add(df_mul(A.m1, fs), df_mul(A.dm, fa[i])));
      A.em[(int64_t)(16 + i) * E + e] = df_to_double(r);
    }
  }
}

// Symmetric storage index of (i, j) in a 4x4 matrix: 0..9.
__host__ __device__ constexpr int sym4(int i, int j) {
  return i <= j ? i * 4 - (i * (i - 1)) / 2 + (j - i) : j * 4 - (j * (j - 1)) / 2 + (i - j);
}

// P1 diffusion + source (+ consistent mass) in closed form: with P1
// coordinates the gradients are the cofactor columns over detJ, so
//   K_ij = (c_i . kappa c_j) * wsum / |detJ|,   c_4 = -(c_1 + c_2 + c_3)
//   rhs_i = sum_j M_ij f_j - sum_j K_ij t_j,  M_ij = |detJ| * Mref_ij.
// This is the pressure-Laplacian form of the Poisson workloads (an exact
// regrouping of dshape_dot_dshape over the rule).  Writes the 10 unique matrix
// entries (k = sym4(i, j)) and 4 rhs entries (k = 10 + i).
__global__ void __launch_bounds__(256) k_asm_p1_diffusion(AsmArgs A) {
  note_launch();
  const RefTensors& R = *A.ref;
  const double M0 = R.M[0][0], M1 = R.M[0][1];
  // theta*dt folds into the stiffness scale (the reference multiplies the
  // element matrix by dt_theta when |dt_theta| > epsilon)
  const double kscale = R.wsum * (A.use_dt ? A.theta_dt : 0.0) * (A.iso ? A.kappa[0] : 1.0);
  const double rscale = R.wsum * (A.iso ? A.kappa[0] : 1.0);
  const int64_t E = A.E;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.E; e += gridDim.x * blockDim.x) {
    Geo g;
    element_geo(A.X, A.xnd, e, g);
    const double adet = fabs(g.det);
    const double rdet = __drcp_rn(adet);
    double c[4][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
#pragma unroll
      for (int i = 0; i < 3; ++i) c[i][a] = g.cof[a][i];
      c[3][a] = -(c[0][a] + c[1][a] + c[2][a]);
    }
    double kc[4][3];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        if (A.iso) kc[i][a] = c[i][a];
        else kc[i][a] = A.kappa[3 * a + 0] * c[i][0] + A.kappa[3 * a + 1] * c[i][1] + A.kappa[3 * a + 2] * c[i][2];
      }
    const int4 tv = __ldg(reinterpret_cast<const int4*>(A.nd) + e);
    const int tn[4] = {tv.x, tv.y, tv.z, tv.w};
    double G[4][4];  // c_i . kappa c_j (symmetric for symmetric kappa)
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = i; j < 4; ++j) {
        G[i][j] = c[i][0] * kc[j][0] + c[i][1] * kc[j][1] + c[i][2] * kc[j][2];
        G[j][i] = G[i][j];
      }
    const double ks = kscale * rdet;
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = i; j < 4; ++j) {
        double m = G[i][j] * ks;
        if (A.have_mass) m += adet * (i == j ? M0 : M1);
        A.em[(int64_t)sym4(i, j) * E + e] = m;
      }
    double fsum = 0.0, fe[4] = {0.0, 0.0, 0.0, 0.0};
    if (A.have_src) {
#pragma unroll
      for (int i = 0; i < 4; ++i) fe[i] = __ldg(A.f + tn[i]);
      fsum = (fe[0] + fe[1]) + (fe[2] + fe[3]);
    }
    double Te[4] = {0.0, 0.0, 0.0, 0.0};
    if (A.t) {
#pragma unroll
      for (int i = 0; i < 4; ++i) Te[i] = __ldg(A.t + tn[i]);
    }
    const double rs = rscale * rdet;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      double r = 0.0;
      if (A.have_src) r = adet * (M1 * fsum + (M0 - M1) * fe[i]);
      if (A.t) r -= (G[i][0] * Te[0] + G[i][1] * Te[1] + G[i][2] * Te[2] + G[i][3] * Te[3]) * rs;
      A.em[(int64_t)(10 + i) * E + e] = r;
    }
  }
}

// P1 diffusion + source (+ consistent mass) in double-float arithmetic: the
// same closed form as k_asm_p1_diffusion with the FP64 pipe used only for the
// nine coordinate differences J(a,b) = x_b - x_4 (one rounding, as the
// reference's matmul with the 0/+-1 entries of dn).  Each difference is split
// exactly into two floats, and cofactors, determinant, reciprocal, the Gram
// products c_i . kappa c_j (isotropic or diagonal kappa), the mass and the
// source integral run on the FP32 pipes with error-free transformations.  The
// rows of the Gram matrix of c_1..c_4 sum to zero (c_4 = -(c_1+c_2+c_3)), so
// only six products are formed.  Output: the 10 unique matrix entries and 4
// rhs entries per element as (hi, lo) float pairs.
struct DfArgs {
  int32_t E;
  const int32_t* nd;
  const int32_t* xnd;
  const double* X;
  const double* t;
  const double* f;
  float2* em;
  df kscale;     // wsum * theta*dt (* kappa if isotropic)
  df rscale;     // wsum (* kappa if isotropic): operator scale of the rhs t-term
  df kdiag[3];   // diagonal kappa (ones if isotropic)
  df m0, m1;     // reference mass entries (diagonal, off-diagonal)
  int have_mass, have_src, aniso;
  // element pass over record positions [p0, E): position q holds element
  // perm[q] (identity when perm is null)
  const int32_t* perm;
  int32_t p0;
};

// Specialised on the term set (consistent mass, source, old field t,
// diagonal kappa) so that each instance carries only its own work.
// Element record: four row slices, slice a = {K_a0, K_a1 | K_a2, r_a} as
// double-float pairs (32 B, one sector), plus {ms, 0} with a mass term (48
// B), where ms = |detJ| (m0 + 3 m1) is the row sum of the element mass
// matrix: K_a3 = ms - (K_a0 + K_a1 + K_a2) because the stiffness rows sum to
// zero.  The records of a warp's 32 consecutive elements are one contiguous
// chunk: each thread stages its float4s in shared memory and the warp writes
// the chunk with coalesced 16-byte stores (blockDim/32 x 4 or 6 kB of
// dynamic shared memory).
//
// One element of the P1 double-float pass: its record (4 row slices) into rec.
// The element's inputs: vertex coordinates, and the source and old-field
// values at its nodes.  (Loading them one element ahead measured no faster at
// 128^3: the registers it holds cost a quarter of the resident warps.)
struct P1In {
  double x[4][3];
  double f[4];
  double t[4];
};

template <bool SRC, bool TF>
__device__ __forceinline__ void p1_df_load(const DfArgs& A, int e, P1In& in) {
  const int4 v = __ldg(reinterpret_cast<const int4*>(A.xnd) + e);
  const int vi[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int a = 0; a < 3; ++a) in.x[i][a] = __ldg(A.X + (uint32_t)(3 * vi[i] + a));
  if (SRC || TF) {
    const int4 tv = __ldg(reinterpret_cast<const int4*>(A.nd) + e);
    const int tn[4] = {tv.x, tv.y, tv.z, tv.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (SRC) in.f[i] = __ldg(A.f + tn[i]);
      if (TF) in.t[i] = __ldg(A.t + tn[i]);
    }
  }
}

// The same loads from connectivity already in registers (xv: vertices, tv:
// field nodes), for the element pass that fetches the next element's
// connectivity one iteration ahead.
template <bool SRC, bool TF>
__device__ __forceinline__ void p1_df_load_from(const DfArgs& A, int4 xv, int4 tv, P1In& in) {
  const int vi[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int a = 0; a < 3; ++a) in.x[i][a] = __ldg(A.X + (uint32_t)(3 * vi[i] + a));
  if (SRC || TF) {
    const int tn[4] = {tv.x, tv.y, tv.z, tv.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      if (SRC) in.f[i] = __ldg(A.f + tn[i]);
      if (TF) in.t[i] = __ldg(A.t + tn[i]);
    }
  }
}

template <bool MASS, bool SRC, bool TF, bool ANISO>
__device__ __forceinline__ void p1_df_element(const DfArgs& A, const P1In& in, float4* rec) {
  constexpr int SL = MASS ? 3 : 2;  // float4 per row slice
  const auto& x = in.x;
  df J[3][3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
#pragma unroll
    for (int b = 0; b < 3; ++b) J[a][b] = df_from_double(x[b][a] - x[3][a]);
  df cof[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, k1 = (k + 1) % 3, k2 = (k + 2) % 3;
      cof[i][k] = df_mul_sub_mul(J[i1][k1], J[i2][k2], J[i2][k1], J[i1][k2]);
    }
  const df det = df_dot3(J[0][0], cof[0][0], J[1][0], cof[1][0], J[2][0], cof[2][0]);
  const df adet = df_abs(det);
  const df rdet = df_rcp(adet);
  // gradient directions c_i = column i of cof; kappa applied to the second factor
  df kc[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int a = 0; a < 3; ++a) kc[i][a] = ANISO ? df_mul(A.kdiag[a], cof[a][i]) : cof[a][i];
  df G[4][4];
#pragma unroll
  for (int i = 0; i < 3; ++i)
#pragma unroll
    for (int j = i; j < 3; ++j) {
      G[i][j] = df_dot3(cof[0][i], kc[j][0], cof[1][i], kc[j][1], cof[2][i], kc[j][2]);
      G[j][i] = G[i][j];
    }
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    G[i][3] = df_neg(df_add(df_add(G[i][0], G[i][1]), G[i][2]));
    G[3][i] = G[i][3];
  }
  G[3][3] = df_neg(df_add(df_add(G[0][3], G[1][3]), G[2][3]));
  const df ks = df_mul(A.kscale, rdet);
  df madet0 = {0.0f, 0.0f}, madet1 = {0.0f, 0.0f};
  if (MASS) {
    madet0 = df_mul(adet, A.m0);
    madet1 = df_mul(adet, A.m1);
  }
  df K[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = i; j < 4; ++j) {
      df m = df_mul(G[i][j], ks);
      if (MASS) m = df_add(m, i == j ? madet0 : madet1);
      K[i][j] = m;
      K[j][i] = m;
    }
  df r[4] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
  if (SRC) {
    df fe[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) fe[i] = df_from_double(in.f[i]);
    const df fsum = df_add(df_add(fe[0], fe[1]), df_add(fe[2], fe[3]));
    const df q1 = df_mul(df_mul(adet, A.m1), fsum);
    const df q2 = df_mul(adet, df_sub(A.m0, A.m1));
#pragma unroll
    for (int i = 0; i < 4; ++i) r[i] = df_add(q1, df_mul(q2, fe[i]));
  }
  if (TF) {
    df te[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) te[i] = df_from_double(in.t[i]);
    const df rs = df_mul(A.rscale, rdet);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      df s = df_add(df_dot3(G[i][0], te[0], G[i][1], te[1], G[i][2], te[2]), df_mul(G[i][3], te[3]));
      r[i] = df_sub(r[i], df_mul(s, rs));
    }
  }
  df ms = {0.0f, 0.0f};
  if (MASS) ms = df_add(madet0, df_add(madet1, df_add(madet1, madet1)));
  // row 3 (b < 3) as the row pass rebuilds column 3 of rows 0..2, so that
  // K_3b and K_b3 are the same double-float value (an exactly symmetric matrix)
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    df k3 = df_neg(df_add(df_add(K[b][0], K[b][1]), K[b][2]));
    if (MASS) k3 = df_add(k3, ms);
    K[3][b] = k3;
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    rec[SL * i + 0] = make_float4(K[i][0].hi, K[i][0].lo, K[i][1].hi, K[i][1].lo);
    rec[SL * i + 1] = make_float4(K[i][2].hi, K[i][2].lo, r[i].hi, r[i].lo);
    if (MASS) rec[SL * i + 2] = make_float4(ms.hi, ms.lo, 0.0f, 0.0f);
  }
}

template <bool MASS, bool SRC, bool TF, bool ANISO>
__global__ void __launch_bounds__(256) k_asm_p1_diffusion_df(DfArgs A) {
  note_launch();
  extern __shared__ float4 stage_all[];
  const int lane = threadIdx.x & 31;
  constexpr int SL = MASS ? 3 : 2;  // float4 per row slice
  constexpr int NREC = 4 * SL;      // float4 per element record
  float4* stage = stage_all + (threadIdx.x >> 5) * (32 * (NREC + 1));
  const int stride = gridDim.x * blockDim.x;
  // the connectivity of the element after this one is fetched while this one
  // is computed (one dependent load round trip fewer per element)
  int4 xv = make_int4(0, 0, 0, 0), tv = xv;
  auto fetch = [&](int e) {
    const int ee = A.perm ? __ldg(A.perm + e) : e;
    xv = __ldg(reinterpret_cast<const int4*>(A.xnd) + ee);
    if (SRC || TF) tv = __ldg(reinterpret_cast<const int4*>(A.nd) + ee);
  };
  int base = A.p0 + blockIdx.x * blockDim.x + (threadIdx.x & ~31);
  if (base + lane < A.E) fetch(base + lane);
  for (; base < A.E; base += stride) {
    const int e = base + lane;
    const int4 cxv = xv, ctv = tv;
    if (base + stride + lane < A.E) fetch(base + stride + lane);
    if (e < A.E) {
      P1In in;
      p1_df_load_from<SRC, TF>(A, cxv, ctv, in);
      p1_df_element<MASS, SRC, TF, ANISO>(A, in, stage + lane * (NREC + 1));
    }
    __syncwarp();
    float4* out = reinterpret_cast<float4*>(A.em) + (uint32_t)base * NREC;
    const int nvalid = min(32, A.E - base) * NREC;
#pragma unroll
    for (int k = 0; k < NREC; ++k) {
      const int idx = k * 32 + lane;
      if (idx < nvalid) out[idx] = stage[stage_pos<NREC>(k, lane)];
    }
    __syncwarp();
  }
}

// P2 diffusion + source (+ consistent mass) in double-float.  With P1
// coordinates the reference gradients are constant per element, so
//   K_ij = theta dt / |detJ| * sum_k Q_k S_ij,k (+ |detJ| Mref_ij),
//   Q = cof^T kappa cof (6 symmetric components),
//   S_ij,k = sum_g w dN_i/dL_a dN_j/dL_b over the rule, symmetrised in (a, b),
//   rhs_i = |detJ| sum_j Mref_ij f_j - 1/|detJ| sum_j (sum_k Q_k S_ij,k) t_j,
// an exact regrouping of dshape_dot_dshape / dshape_tensor_dshape
// (FETools.F90:391,668) over the quadrature rule, as for P1.  The tables
// (55 symmetric pairs) travel as kernel parameters.  Each element writes ten
// row slices {K_i0..K_i9, r_i, 0} of double-float pairs (96 B each), stored
// slice-major (slice i of element e at i E + e) so that a warp's slices i
// form one contiguous run written with coalesced stores.
struct DfP2Args {
  int32_t E;
  const int32_t* nd;   // P2 connectivity, 10 per element
  const int32_t* xnd;  // P1 coordinate connectivity
  const double* X;
  const double* t;
  const double* f;
  float4* em;
  df S[55][6];
  df M[55];
  df qs;        // theta*dt (zero when the dt factor is not applied)
  df kdiag[3];  // diagonal kappa (isotropic: kappa in every entry)
  int have_mass, have_src;
};

__host__ __device__ constexpr int sym10(int i, int j) {
  return i <= j ? i * 10 - (i * (i - 1)) / 2 + (j - i) : j * 10 - (j * (j - 1)) / 2 + (i - j);
}

// sum_k a_k b_k of double-float values: exact leading products (FMA
// TwoProduct) summed by TwoSum, all error terms in one float, one
// renormalisation.
template <int K>
__device__ __forceinline__ df df_dot(const df* a, const df* b) {
  float s = a[0].hi * b[0].hi;
  float e = fmaf(a[0].hi, b[0].hi, -s);
  e = fmaf(a[0].hi, b[0].lo, e);
  e = fmaf(a[0].lo, b[0].hi, e);
#pragma unroll
  for (int k = 1; k < K; ++k) {
    const float p = a[k].hi * b[k].hi;
    float ep = fmaf(a[k].hi, b[k].hi, -p);
    ep = fmaf(a[k].hi, b[k].lo, ep);
    ep = fmaf(a[k].lo, b[k].hi, ep);
    const df t = df_two_sum(s, p);
    s = t.hi;
    e += t.lo + ep;
  }
  return df_fast_two_sum(s, e);
}

constexpr int kP2Threads = 128;

__global__ void __launch_bounds__(kP2Threads) k_asm_p2_diffusion_df(DfP2Args A) {
  note_launch();
  __shared__ float4 stage_all[kP2Threads / 32][32 * 7];  // one 96-B slice per lane and warp, padded
  extern __shared__ float2 p2_dots[];      // [45][kP2Threads]: the strict upper d_ij
  const int lane = threadIdx.x & 31;
  float4* stage = stage_all[threadIdx.x >> 5];
  float2* dots = p2_dots + threadIdx.x;
  for (int base = blockIdx.x * blockDim.x + (threadIdx.x & ~31); base < A.E; base += gridDim.x * blockDim.x) {
    // lanes past the last element compute on element base (their slices are
    // not stored)
    const int e = base + lane < A.E ? base + lane : base;
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
    df cof[3][3];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        const int i1 = (i + 1) % 3, i2 = (i + 2) % 3, k1 = (k + 1) % 3, k2 = (k + 2) % 3;
        cof[i][k] = df_mul_sub_mul(J[i1][k1], J[i2][k2], J[i2][k1], J[i1][k2]);
      }
    const df det = df_dot3(J[0][0], cof[0][0], J[1][0], cof[1][0], J[2][0], cof[2][0]);
    const df adet = df_abs(det);
    const df rdet = df_rcp(adet);
    // Q_ab = sum_c cof_ca kappa_c cof_cb in the order 00, 11, 22, 01, 02, 12
    const int qa[6] = {0, 1, 2, 0, 0, 1}, qb[6] = {0, 1, 2, 1, 2, 2};
    df qo[6], qk[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      const int a = qa[k], b = qb[k];
      const df q = df_dot3(cof[0][a], df_mul(A.kdiag[0], cof[0][b]), cof[1][a], df_mul(A.kdiag[1], cof[1][b]),
                           cof[2][a], df_mul(A.kdiag[2], cof[2][b]));
      qo[k] = df_mul(q, rdet);    // operator: 1/|detJ| Q
      qk[k] = df_mul(qo[k], A.qs);  // matrix: theta dt/|detJ| Q
    }
    int tn[10];
    {
      // 10 ints per element: element e starts at 40 e bytes, 8-byte aligned
      const int2* nd2 = reinterpret_cast<const int2*>(A.nd + (uint32_t)e * 10u);
#pragma unroll
      for (int k = 0; k < 5; ++k) {
        const int2 w = __ldg(nd2 + k);
        tn[2 * k] = w.x;
        tn[2 * k + 1] = w.y;
      }
    }
    df fe[10], te[10];
#pragma unroll
    for (int j = 0; j < 10; ++j) {
      fe[j] = A.have_src ? df_mul(adet, df_from_double(__ldg(A.f + tn[j]))) : df{0.0f, 0.0f};
      te[j] = A.t ? df_from_double(__ldg(A.t + tn[j])) : df{0.0f, 0.0f};
    }
    // slice i of the warp's 32 elements is one contiguous run of the
    // slice-major records: stage it and store it with coalesced 16-B stores
    const int nvalid = min(32, A.E - base) * 6;
#pragma unroll 1
    for (int i = 0; i < 10; ++i) {
      // d_ij = q . S_ij is symmetric: row i computes j >= i and keeps j > i
      // for the later rows in its own column of shared memory
      df K[10];
      df tsum = {0.0f, 0.0f};
#pragma unroll
      for (int j = 0; j < 10; ++j) {
        df d;
        if (j >= i) {
          d = df_dot<6>(A.t ? qo : qk, A.S[sym10(i, j)]);
          if (j > i) {
            const int u = i * 9 - i * (i - 1) / 2 + (j - i - 1);
            dots[u * kP2Threads] = make_float2(d.hi, d.lo);
          }
        } else {
          const int u = j * 9 - j * (j - 1) / 2 + (i - j - 1);
          const float2 w = dots[u * kP2Threads];
          d = {w.x, w.y};
        }
        if (A.t) {
          K[j] = df_mul(d, A.qs);
          tsum = df_add(tsum, df_mul(d, te[j]));
        } else {
          K[j] = d;
        }
        if (A.have_mass) K[j] = df_add(K[j], df_mul(adet, A.M[sym10(i, j)]));
      }
      df r = {0.0f, 0.0f};
      if (A.have_src) {
        df mrow[10];
#pragma unroll
        for (int j = 0; j < 10; ++j) mrow[j] = A.M[sym10(i, j)];
        r = df_dot<10>(mrow, fe);
      }
      if (A.t) r = df_sub(r, tsum);
      float4* rec = stage + lane * 7;
#pragma unroll
      for (int k = 0; k < 5; ++k)
        rec[k] = make_float4(K[2 * k].hi, K[2 * k].lo, K[2 * k + 1].hi, K[2 * k + 1].lo);
      rec[5] = make_float4(r.hi, r.lo, 0.0f, 0.0f);
      __syncwarp();
      float4* out = A.em + ((uint32_t)i * (uint32_t)A.E + (uint32_t)base) * 6u;
#pragma unroll
      for (int k = 0; k < 6; ++k) {
        const int idx = k * 32 + lane;
        if (idx < nvalid) out[idx] = stage[stage_pos<6>(k, lane)];
      }
      __syncwarp();
    }
  }
}

// Row pass: thread per CSR row; contributions of the row's elements are added
// in the colour order of ne_col and the row is written once.  Accumulators
// and the row's column indices live in shared memory for rows up to RMAX
// entries; longer rows accumulate in place in val (the row belongs to this
// thread alone).  A column missing from the pattern is csr_addto's
// "outside sparsity pattern" error.
struct PullArgs {
  int32_t N, E;
  const int32_t* ne_ptr;
  const int32_t* ne_col;
  const int32_t* ne_rec;  // fused P1 pass: record slice of every ne_col incidence
  const uint32_t* ne_pos;
  const int32_t* nd;
  const int32_t* findrm;
  const int32_t* colm;
  const double* em;
  double* val;
  double* rhs;
  ErrWord* err;
  int coalesce;  // P1 double-float rows: warp-cooperative stores of val (val in host memory)
  int32_t row0;  // P1 double-float rows: the pass covers rows [row0, N)
};

// Double-float version of the row pass over the P1 element records: the
// slice of (element, local row a) gives K_a0..K_a2 and r_a, and K_a3 is the
// row's mass sum minus their sum; each row accumulates in double-float
// (shared memory, or in val for rows longer than RMAX) and converts every
// entry to double once.
// One row per lane of the P1 double-float row pass; all 32 lanes of a warp
// call it together for 32 consecutive rows (live = false past the last row).
// FUSED: the record slice of each incidence comes from P.ne_rec (records in
// element-item order); otherwise it is (element, local row) of P.ne_col.
// The fused pass reads records through L1 (ld.global.ca, not the read-only
// ld.global.nc path) although other blocks of the same kernel wrote them: an
// item's records are one 128-B aligned block (256 records of 128 or 192 B),
// written by one block, a row item touches an item's lines only after the
// item is complete, and L1 starts every kernel empty, so no L1 line can hold
// data older than the item that wrote it.  The warp
// stores each row's entries; with P.coalesce (val in mapped host memory) the
// warp stores its rows' entries, one contiguous range of val, with coalesced
// stores instead.
template <int THREADS, int RMAX, bool MASS, bool FUSED>
__device__ __forceinline__ void p1_df_row(const PullArgs& P, int row, bool live, float2* acc, int t) {
  constexpr int SL = MASS ? 3 : 2;  // float4 per row slice
  const float4* rec = reinterpret_cast<const float4*>(P.em);
  const int lane = t & 31;
  int base = 0, L = 0;
  if (live) {
    base = __ldg(P.findrm + row);
    L = __ldg(P.findrm + row + 1) - base;
  }
  const bool in_smem = L <= RMAX;
  if (in_smem) {
    for (int k = 0; k < L; ++k) acc[k * THREADS + t] = make_float2(0.0f, 0.0f);
  } else {
    for (int k = 0; k < L; ++k) P.val[base + k] = 0.0;
  }
  df r = {0.0f, 0.0f};
  const int ib = live ? __ldg(P.ne_ptr + row) : 0, ie = live ? __ldg(P.ne_ptr + row + 1) : 0;
  // incidences in groups of four: all index and record loads of a group are
  // issued before any accumulation (memory-level parallelism), and the next
  // group's indices are loaded while this group's records are in flight
  // (software pipelining: one dependent round trip per group instead of
  // two); the adds run in the group's order, so the colour order of the sum
  // is kept
  const int32_t* incl = FUSED ? P.ne_rec : P.ne_col;
  int ninc[4];
  uint32_t npw[4];
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const bool ok = ib + u < ie;
    ninc[u] = ok ? __ldg(incl + ib + u) : 0;
    npw[u] = ok ? __ldg(P.ne_pos + ib + u) : 0u;
  }
  for (int q0 = ib; q0 < ie; q0 += 4) {
    int inc[4];
    uint32_t pw[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      inc[u] = ninc[u];
      pw[u] = npw[u];
    }
    float4 q[4][SL];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const uint32_t slice = FUSED ? (uint32_t)inc[u] : (uint32_t)(((inc[u] >> 4) << 2) | (inc[u] & 15));
      const uint32_t ri = (uint32_t)SL * slice;
      if (!MASS && !FUSED) {
        // a 32-B slice (32-B aligned) in one 256-bit load
        if (q0 + u < ie) ldg256(rec + ri, q[u][0], q[u][1]);
        else q[u][0] = q[u][1] = make_float4(0.f, 0.f, 0.f, 0.f);
      } else {
#pragma unroll
        for (int k = 0; k < SL; ++k) {
          if (q0 + u < ie) q[u][k] = FUSED ? __ldca(rec + ri + k) : __ldg(rec + ri + k);
          else q[u][k] = make_float4(0.f, 0.f, 0.f, 0.f);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const bool ok = q0 + 4 + u < ie;
      ninc[u] = ok ? __ldg(incl + q0 + 4 + u) : 0;
      npw[u] = ok ? __ldg(P.ne_pos + q0 + 4 + u) : 0u;
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (q0 + u >= ie) break;
      df v[4];
      v[0] = {q[u][0].x, q[u][0].y};
      v[1] = {q[u][0].z, q[u][0].w};
      v[2] = {q[u][1].x, q[u][1].y};
      v[3] = df_neg(df_add(df_add(v[0], v[1]), v[2]));
      if (MASS) v[3] = df_add(v[3], {q[u][SL - 1].x, q[u][SL - 1].y});
      if (in_smem) {
        // an element's four nodes are four different columns of the row, so
        // the four accumulators are read together, then written together
        // (one shared-memory round trip per incidence instead of four)
        int pos[4];
        float2 c[4];
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          pos[b] = ((pw[u] >> (8 * b)) & 0xffu) * THREADS + t;
          c[b] = acc[pos[b]];
        }
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const df sum = df_add({c[b].x, c[b].y}, v[b]);
          acc[pos[b]] = make_float2(sum.hi, sum.lo);
        }
      } else {
#pragma unroll
        for (int b = 0; b < 4; ++b) P.val[base + ((pw[u] >> (8 * b)) & 0xffu)] += df_to_double(v[b]);
      }
      r = df_add(r, {q[u][1].z, q[u][1].w});
    }
  }
  if (!P.coalesce) {
    if (in_smem)
      for (int k = 0; k < L; ++k) {
        const float2 c = acc[k * THREADS + t];
        P.val[base + k] = df_to_double({c.x, c.y});
      }
  } else {
    __syncwarp();
    // the warp's rows [r0, r0 + 32) hold val[start, end): lane j of each pass
    // stores entry start + 32 m + j, found in the accumulators of its row's lane
    const int start = __shfl_sync(0xffffffffu, base, 0);
    const int nlive = __popc(__ballot_sync(0xffffffffu, live));
    const int end = nlive ? __shfl_sync(0xffffffffu, base + L, nlive - 1) : start;
    const unsigned smem_rows = __ballot_sync(0xffffffffu, in_smem);
    const int wt = t & ~31;  // thread index of lane 0
    for (int p0 = start; p0 < end; p0 += 32) {
      const int p = p0 + lane;
      // owner: the last lane whose row starts at or before p (5 halvings)
      int lo = 0;
#pragma unroll
      for (int step = 16; step > 0; step >>= 1) {
        const int cand = lo + step;
        const int cb = __shfl_sync(0xffffffffu, base, cand < nlive ? cand : 0);
        if (cand < nlive && cb <= p) lo = cand;
      }
      const int ob = __shfl_sync(0xffffffffu, base, lo);
      if (p < end && ((smem_rows >> lo) & 1u)) {
        const float2 c = acc[(p - ob) * THREADS + wt + lo];
        P.val[p] = df_to_double({c.x, c.y});
      }
    }
  }
  if (live) P.rhs[row] = df_to_double(r);
}

// PERM: records in the fused pass's element order (slices from P.ne_rec).
template <int THREADS, int RMAX, bool MASS, bool PERM>
__global__ void __launch_bounds__(THREADS) k_rows_pull_df(PullArgs P) {
  note_launch();
  extern __shared__ unsigned char smem_raw[];
  float2* acc = reinterpret_cast<float2*>(smem_raw);  // [RMAX][THREADS]
  for (int r0 = P.row0 + blockIdx.x * THREADS; r0 < P.N; r0 += gridDim.x * THREADS) {
    const int row = r0 + threadIdx.x;
    p1_df_row<THREADS, RMAX, MASS, PERM>(P, row, row < P.N, acc, threadIdx.x);
  }
}

// ----------------------------------------- fused P1 element and row pass --
// One persistent kernel over a work queue of element items (256 elements in
// the order of their highest field node, one per thread) and row items (256
// rows).  Element items are counted done per group of kFzGroup items; a row
// item waits, with a bounded spin, until the groups holding the element items
// of its incidences are complete (threadfence + atomic add on one side,
// acquire loads on the other), then sums its rows exactly as the row pass
// does, in colour order: the result is bit-identical to the two kernels.
// Row items follow the element items they need at a distance of about three
// resident waves, so the records they read were written moments earlier and
// are still in L2.  Every group a row item waits for holds only items dequeued before
// it by running blocks, so the queue always drains; a wait that runs out sets
// FL_ERR_TIMEOUT.
struct FusedArgs {
  int32_t nitems;
  int32_t ne;            // element items
  const int32_t* items;  // k >= 0: element item k; -(j+1): row item j
  const int32_t* perm;   // elements by (highest field node, element id)
  const int32_t* need;   // per row item: [first, last] element item it reads
  int32_t* gdone;        // per group of kFzGroup element items: items done
  int32_t* ctl;          // [0] queue head
  ErrWord* err;
  unsigned spin_limit;   // polls of one counter before giving up
  int32_t withhold;      // failure-injection test: this group never counts complete
};
constexpr int kFzItem = 256;             // elements or rows per item = threads per block
constexpr int kFzGroup = 64;             // element items per completion counter
constexpr unsigned kFzSpin = 1u << 22;   // polls of one counter before giving up
constexpr int64_t kCkBytes = 4 << 20;    // pipelined host output: val bytes per row chunk
constexpr int64_t kCkMax = 16;           // and at most this many chunks

template <bool MASS, bool SRC, bool TF, bool ANISO>
__global__ void __launch_bounds__(kFzItem) k_asm_p1_fused(DfArgs A, PullArgs P, FusedArgs F) {
  note_launch();
  extern __shared__ float4 fz_smem[];
  constexpr int SL = MASS ? 3 : 2, NREC = 4 * SL;
  __shared__ int s_item;
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  float4* stage = fz_smem + w * (32 * (NREC + 1));
  float2* acc = reinterpret_cast<float2*>(fz_smem);  // [16][kFzItem]
  for (;;) {
    if (t == 0) s_item = atomicAdd(F.ctl, 1);
    __syncthreads();
    const int it = s_item;
    if (it >= F.nitems) break;
    const int code = __ldg(F.items + it);
    if (code >= 0) {
      const int base = code * kFzItem + w * 32;  // this warp's 32 consecutive positions
      if (base < A.E) {
        const int pp = base + lane;
        if (pp < A.E) {
          P1In in;
          p1_df_load<SRC, TF>(A, __ldg(F.perm + pp), in);
          p1_df_element<MASS, SRC, TF, ANISO>(A, in, stage + lane * (NREC + 1));
        }
        __syncwarp();
        float4* out = reinterpret_cast<float4*>(A.em) + (uint32_t)base * NREC;
        const int nvalid = min(32, A.E - base) * NREC;
#pragma unroll
        for (int k = 0; k < NREC; ++k) {
          const int idx = k * 32 + lane;
          if (idx < nvalid) out[idx] = stage[stage_pos<NREC>(k, lane)];
        }
      }
      __syncthreads();
      if (t == 0) {
        __threadfence();
        atomicAdd(F.gdone + code / kFzGroup, 1);
      }
    } else {
      const int j = -code - 1;
      if (t == 0) {
        const int first = __ldg(F.need + 2 * j), last = __ldg(F.need + 2 * j + 1);
        unsigned spins = 0;
        for (int g = first / kFzGroup; last >= 0 && g <= last / kFzGroup; ++g) {
          const int target = min(kFzGroup, F.ne - g * kFzGroup) + (g == F.withhold ? 1 : 0);
          while (ld_acquire(F.gdone + g) < target) {
            if (++spins > F.spin_limit) break;
            __nanosleep(64);
          }
          if (spins > F.spin_limit) {
            set_err(F.err, FL_ERR_TIMEOUT, j);
            break;
          }
        }
      }
      __syncthreads();
      const int row = j * kFzItem + t;
      p1_df_row<kFzItem, 16, MASS, true>(P, row, row < P.N, acc, t);
    }
    __syncthreads();
  }
}

// Plan of the fused pass (once per mesh): element order, record slice of
// every incidence, the row items' needs and the queue.
__global__ void k_fz_maxv(int32_t E, const int32_t* __restrict__ nd, int32_t* __restrict__ maxv) {
  note_launch();
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < E; e += gridDim.x * blockDim.x) {
    const int4 v = reinterpret_cast<const int4*>(nd)[e];
    maxv[e] = max(max(v.x, v.y), max(v.z, v.w));
  }
}

// pass 0: count the elements whose highest node is v; pass 1: place them in
// ascending element order (the incidence list of v is ascending)
__global__ void k_fz_place(int32_t N, const int32_t* __restrict__ ne_ptr, const int32_t* __restrict__ ne,
                           const int32_t* __restrict__ maxv, int32_t* __restrict__ cnt,
                           const int32_t* __restrict__ off, int32_t* __restrict__ perm, int32_t* __restrict__ pos,
                           int pass) {
  note_launch();
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) {
    int c = 0;
    for (int q = ne_ptr[v]; q < ne_ptr[v + 1]; ++q) {
      const int e = ne[q] >> 4;
      if (maxv[e] != v) continue;
      if (pass) {
        perm[off[v] + c] = e;
        pos[e] = off[v] + c;
      }
      ++c;
    }
    if (!pass) cnt[v] = c;
  }
}

__global__ void k_fz_rec(int32_t N, const int32_t* __restrict__ ne_ptr, const int32_t* __restrict__ ne_col,
                         const int32_t* __restrict__ pos, int32_t* __restrict__ rec, int32_t* __restrict__ rowrange) {
  note_launch();
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < N; v += gridDim.x * blockDim.x) {
    int mx = -1, mn = INT_MAX;
    for (int q = ne_ptr[v]; q < ne_ptr[v + 1]; ++q) {
      const int inc = ne_col[q];
      const int p = pos[inc >> 4];
      rec[q] = 4 * p + (inc & 15);
      mx = max(mx, p);
      mn = min(mn, p);
    }
    rowrange[2 * v] = mn;
    rowrange[2 * v + 1] = mx;
  }
}

static int fused_plan(fl_mesh_t* m, cudaStream_t s) {
  if (m->fz_state != 0) return FL_OK;
  m->fz_state = -1;
  const int N = m->N, E = m->E;
  const int64_t ninc = (int64_t)4 * E;
  DevBuf<int32_t> maxv, cnt, off, pos, rowmax;
  FL_TRY(maxv.reserve(E));
  FL_TRY(cnt.reserve((size_t)N + 1));
  FL_TRY(off.reserve((size_t)N + 1));
  FL_TRY(pos.reserve(E));
  FL_TRY(rowmax.reserve((size_t)2 * N));
  FL_TRY(m->fz_perm.reserve(E));
  FL_TRY(m->fz_rec.reserve((size_t)ninc));
  k_fz_maxv<<<grid_for(E, 256), 256, 0, s>>>(E, m->ndglno.p, maxv.p);
  k_fz_place<<<grid_for(N, 256), 256, 0, s>>>(N, m->ne_ptr.p, m->ne.p, maxv.p, cnt.p, nullptr, nullptr, nullptr, 0);
  FL_TRY(exclusive_scan_i32(cnt.p, off.p, N, s));
  k_fz_place<<<grid_for(N, 256), 256, 0, s>>>(N, m->ne_ptr.p, m->ne.p, maxv.p, nullptr, off.p, m->fz_perm.p, pos.p,
                                              1);
  k_fz_rec<<<grid_for(N, 256), 256, 0, s>>>(N, m->ne_ptr.p, m->ne_col.p, pos.p, m->fz_rec.p, rowmax.p);
  FL_TRY_CUDA(cudaGetLastError());
  std::vector<int32_t> hmax((size_t)2 * N);
  int32_t placed = 0;
  FL_TRY_CUDA(cudaMemcpyAsync(hmax.data(), rowmax.p, sizeof(int32_t) * 2 * N, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaMemcpyAsync(&placed, off.p + N, sizeof(int32_t), cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  if (placed != E) {
    set_error("fused pass plan: %d of %d elements placed", placed, E);
    return FL_ERR_ARG;
  }
  // Row chunks of the pipelined host-output assembly: about kCkBytes of val
  // each (at most kCkMax), the first a quarter of the others so that the
  // host link starts early; chunk k needs the element positions up to the
  // highest one its rows (and all earlier rows) read, rounded up to a whole
  // warp of records, and the field values up to the highest node of those
  // elements (positions are in ascending highest-node order).
  m->ck_rows.clear();
  m->ck_elem.clear();
  m->ck_val.clear();
  m->ck_node.clear();
  const int64_t K = std::min<int64_t>(kCkMax, m->nnz * (int64_t)sizeof(double) / kCkBytes);
  const int64_t Q = 4 * K - 3;  // quarter chunks
  if (K >= 2 && N >= Q) {
    std::vector<int32_t> hf((size_t)N + 1);
    FL_TRY_CUDA(cudaMemcpyAsync(hf.data(), m->findrm.p, sizeof(int32_t) * ((size_t)N + 1), cudaMemcpyDeviceToHost, s));
    FL_TRY_CUDA(cudaStreamSynchronize(s));
    m->ck_rows.push_back(0);
    m->ck_elem.push_back(0);
    m->ck_val.push_back(hf[0]);
    m->ck_node.push_back(0);
    int32_t need = 0;
    int64_t k = 1;
    for (int32_t i = 0; i < N; ++i) {
      need = std::max(need, hmax[2 * (size_t)i + 1] + 1);
      const int32_t rk = (int32_t)((int64_t)N * (4 * k - 3) / Q);
      if (i + 1 == rk) {
        m->ck_rows.push_back(rk);
        m->ck_elem.push_back(k == K ? E : std::min(E, std::max(m->ck_elem.back(), (need + 31) & ~31)));
        m->ck_val.push_back(hf[rk]);
        ++k;
      }
    }
    for (k = 1; k <= K; ++k) {
      int32_t node = 0;
      const int32_t q = m->ck_elem[k];
      if (k == K) {
        node = N;
      } else if (q > 0) {
        int32_t e = 0;
        FL_TRY_CUDA(cudaMemcpy(&e, m->fz_perm.p + (q - 1), sizeof(int32_t), cudaMemcpyDeviceToHost));
        FL_TRY_CUDA(cudaMemcpy(&node, maxv.p + e, sizeof(int32_t), cudaMemcpyDeviceToHost));
        node += 1;
      }
      m->ck_node.push_back(std::max(m->ck_node.back(), node));
    }
  }
  const int nE = (E + kFzItem - 1) / kFzItem, nR = (N + kFzItem - 1) / kFzItem;
  // need[j] = number of element items up to the last one row item j reads;
  // range[j] = its first and last element item (-1, -1 for rows without elements)
  std::vector<int32_t> need(nR), order(nR), range((size_t)2 * nR);
  for (int j = 0; j < nR; ++j) {
    int mx = -1, mn = INT_MAX;
    for (int i = j * kFzItem; i < std::min(N, (j + 1) * kFzItem); ++i) {
      mx = std::max(mx, hmax[2 * i + 1]);
      mn = std::min(mn, hmax[2 * i]);
    }
    need[j] = mx < 0 ? 0 : mx / kFzItem + 1;
    range[2 * j] = mx < 0 ? -1 : mn / kFzItem;
    range[2 * j + 1] = mx < 0 ? -1 : mx / kFzItem;
    order[j] = j;
  }
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return need[a] < need[b]; });
  // row items trail the element items they need by about three resident waves
  // (at least a completion group, so a group a row item waits for was fully
  // dequeued before it)
  const int per_sm = 4;
  const int lag = std::max(kFzGroup, 3 * num_sms() * per_sm);
  std::vector<int32_t> items;
  items.reserve((size_t)nE + nR);
  size_t r = 0;
  for (int k = 0; k < nE; ++k) {
    items.push_back(k);
    while (r < order.size() && need[order[r]] <= k + 1 - lag) items.push_back(-(order[r++] + 1));
  }
  while (r < order.size()) items.push_back(-(order[r++] + 1));
  const int ng = (nE + kFzGroup - 1) / kFzGroup;
  FL_TRY(m->fz_items.reserve(items.size()));
  FL_TRY(m->fz_need.reserve((size_t)2 * nR));
  FL_TRY(m->fz_ctl.reserve((size_t)1 + ng));
  FL_TRY_CUDA(cudaMemcpyAsync(m->fz_items.p, items.data(), sizeof(int32_t) * items.size(), cudaMemcpyHostToDevice, s));
  FL_TRY_CUDA(cudaMemcpyAsync(m->fz_need.p, range.data(), sizeof(int32_t) * 2 * nR, cudaMemcpyHostToDevice, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));  // host vectors and scratch are released on return
  m->fz_nitems = (int32_t)items.size();
  m->fz_state = 1;
  return FL_OK;
}

template <bool MASS, bool SRC, bool TF, bool ANISO>
static int launch_fused(fl_mesh_t* m, const DfArgs& D, const PullArgs& P, cudaStream_t s) {
  constexpr int NREC = MASS ? 12 : 8;
  const size_t smem = std::max((size_t)(kFzItem / 32) * 32 * (NREC + 1) * sizeof(float4),
                               (size_t)16 * kFzItem * sizeof(float2));
  static bool configured = false;
  if (!configured) {
    FL_TRY_CUDA(cudaFuncSetAttribute(k_asm_p1_fused<MASS, SRC, TF, ANISO>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured = true;
  }
  int per_sm = 0;
  FL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_asm_p1_fused<MASS, SRC, TF, ANISO>, kFzItem,
                                                            smem));
  const int ne = (m->E + kFzItem - 1) / kFzItem, ng = (ne + kFzGroup - 1) / kFzGroup;
  // ctl[0] queue head, ctl[1..ng] group counters: zeroed per call
  const WaitTest& wt = wait_test();
  // about 0.5 us per poll (a 64 ns sleep and an L2 load)
  const unsigned spin = wt.wait_ms > 0.0 ? (unsigned)std::max(1.0, wt.wait_ms * 2000.0) : kFzSpin;
  FusedArgs F{m->fz_nitems, ne, m->fz_items.p, m->fz_perm.p, m->fz_need.p, m->fz_ctl.p + 1, m->fz_ctl.p, m->err.p,
              spin, wt.withhold};
  FL_TRY_CUDA(cudaMemsetAsync(m->fz_ctl.p, 0, sizeof(int32_t) * (1 + ng), s));
  const unsigned g = (unsigned)std::max(1, std::min(m->fz_nitems, num_sms() * std::max(1, per_sm)));
  k_asm_p1_fused<MASS, SRC, TF, ANISO><<<g, kFzItem, smem, s>>>(D, P, F);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

// Row pass of the P2 double-float records: slice (element, local row) =
// 6 float4 {K_a0..K_a9, r_a, 0} at (local row) E + element; the row
// positions of the ten element nodes come from three ne_pos words per
// incidence.  One half-warp per row: in each incidence step
// lane b (0..9) adds K_ab into the slot of node b's column and lane 10 takes
// r_a, so a row's accumulators (shared memory, up to kP2HwSlots entries; longer
// rows add into val) cost one row's worth of shared memory, not one per
// thread, and the row's val range is stored with coalesced stores.  The
// incidences go in colour order and the ten positions of one incidence are
// distinct, so every entry is summed in colour order, as one thread per row
// would.  The next incidence's index and positions are loaded during the
// current step.
constexpr int kP2HwSlots = 128;
constexpr int kP2HwWarps = 8;

__global__ void __launch_bounds__(kP2HwWarps * 32) k_rows_p2_hw(PullArgs P) {
  note_launch();
  // per row: kP2HwSlots accumulators, then the rhs slot and a dummy slot
  __shared__ float2 acc_all[2 * kP2HwWarps][kP2HwSlots + 2];
  const int lane = threadIdx.x & 31, half = lane >> 4, hl = lane & 15;
  const int hw = (threadIdx.x >> 5) * 2 + half;
  float2* acc = acc_all[hw];
  const float2* rec = reinterpret_cast<const float2*>(P.em);  // slices of 12 pairs
  constexpr int kRhs = kP2HwSlots, kDummy = kP2HwSlots + 1;
  const bool val_lane = hl < 10, rhs_lane = hl == 10;
  const int own = rhs_lane ? kRhs : kDummy;  // slot of lanes 10..15
  const int nhw = gridDim.x * 2 * kP2HwWarps;
  const int nsteps = (P.N + nhw - 1) / nhw;  // the same for every half-warp
  for (int it = 0; it < nsteps; ++it) {
    const int row = it * nhw + blockIdx.x * 2 * kP2HwWarps + hw;
    const bool live = row < P.N;
    int base = 0, L = 0, ib = 0, ie = 0;
    if (live) {
      base = __ldg(P.findrm + row);
      L = __ldg(P.findrm + row + 1) - base;
      ib = __ldg(P.ne_ptr + row);
      ie = __ldg(P.ne_ptr + row + 1);
    }
    const bool in_smem = L <= kP2HwSlots;
    if (in_smem) {
      for (int t = hl; t < L; t += 16) acc[t] = make_float2(0.0f, 0.0f);
      if (rhs_lane) acc[kRhs] = make_float2(0.0f, 0.0f);
    } else {
      for (int t = hl; t < L; t += 16) P.val[base + t] = 0.0;
    }
    __syncwarp();
    const int n = ie - ib;
    const int nmax = max(n, __shfl_xor_sync(0xffffffffu, n, 16));
    const bool uniform = __all_sync(0xffffffffu, in_smem);
    df r = {0.0f, 0.0f};
    int inc = 0;
    uint32_t pw = 0u;
    if (n > 0) {
      inc = __ldg(P.ne_col + ib);
      if (val_lane) pw = __ldg(P.ne_pos + (int64_t)ib * 3 + (hl >> 2));
    }
    for (int q = 0; q < nmax; ++q) {
      const bool ok = q < n;
      const uint32_t slice = (uint32_t)(inc & 15) * (uint32_t)P.E + (uint32_t)(inc >> 4);
      // lanes past 10 and steps past the row's end read the slice's first pair
      float2 v = __ldg(rec + 12u * slice + (hl <= 10 ? hl : 0));
      const uint32_t cpw = pw;
      if (q + 1 < n) {
        inc = __ldg(P.ne_col + ib + q + 1);
        if (val_lane) pw = __ldg(P.ne_pos + (int64_t)(ib + q + 1) * 3 + (hl >> 2));
      }
      const int slot = !ok ? kDummy : val_lane ? (int)((cpw >> (8 * (hl & 3))) & 0xffu) : own;
      if (uniform) {
        // every lane adds into its slot (distinct for lanes 0..10)
        const float2 c = acc[slot];
        const df sum = df_add({c.x, c.y}, {v.x, v.y});
        acc[slot] = make_float2(sum.hi, sum.lo);
      } else if (ok && val_lane) {
        if (in_smem) {
          const float2 c = acc[slot];
          const df sum = df_add({c.x, c.y}, {v.x, v.y});
          acc[slot] = make_float2(sum.hi, sum.lo);
        } else {
          P.val[base + slot] += df_to_double({v.x, v.y});
        }
      } else if (ok && rhs_lane) {
        r = df_add(r, {v.x, v.y});
      }
      __syncwarp();
    }
    if (in_smem) {
      for (int t = hl; t < L; t += 16) {
        const float2 c = acc[t];
        P.val[base + t] = df_to_double({c.x, c.y});
      }
      if (uniform && rhs_lane) r = {acc[kRhs].x, acc[kRhs].y};
    }
    if (live && rhs_lane) P.rhs[row] = df_to_double(r);
    __syncwarp();
  }
}

static int launch_rows_p2_hw(const PullArgs& P, cudaStream_t s) {
  int per_sm = 0;
  FL_TRY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_rows_p2_hw, kP2HwWarps * 32, 0));
  const int rows_per_block = 2 * kP2HwWarps;
  const unsigned grid = (unsigned)std::max(
      1, std::min((P.N + rows_per_block - 1) / rows_per_block, num_sms() * std::max(1, per_sm)));
  k_rows_p2_hw<<<grid, kP2HwWarps * 32, 0, s>>>(P);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

template <int THREADS, int RMAX, bool MASS, bool PERM>
static int launch_pull_df(const PullArgs& P, cudaStream_t s) {
  const size_t smem = (size_t)RMAX * THREADS * sizeof(float2);
  static bool configured = false;
  if (!configured) {
    FL_TRY_CUDA(cudaFuncSetAttribute(k_rows_pull_df<THREADS, RMAX, MASS, PERM>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured = true;
  }
  const unsigned grid = (unsigned)((P.N - P.row0 + THREADS - 1) / THREADS);
  if (grid == 0) return FL_OK;
  k_rows_pull_df<THREADS, RMAX, MASS, PERM><<<grid, THREADS, smem, s>>>(P);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

template <int LOC, bool SYM, int THREADS, int RMAX>
__global__ void __launch_bounds__(THREADS) k_rows_pull(PullArgs P) {
  note_launch();
  extern __shared__ unsigned char smem_raw[];
  double* acc = reinterpret_cast<double*>(smem_raw);  // [RMAX][THREADS]
  const int t = threadIdx.x;
  const int64_t E = P.E;
  constexpr int NK = SYM ? LOC * (LOC + 1) / 2 : LOC * LOC;
  constexpr int PW = (LOC + 3) / 4;
  for (int row = blockIdx.x * THREADS + t; row < P.N; row += gridDim.x * THREADS) {
    const int base = __ldg(P.findrm + row), L = __ldg(P.findrm + row + 1) - base;
    const bool in_smem = L <= RMAX;
    if (in_smem) {
      for (int k = 0; k < L; ++k) acc[k * THREADS + t] = 0.0;
    } else {
      for (int k = 0; k < L; ++k) P.val[base + k] = 0.0;
    }
    double r = 0.0;
    const int ib = __ldg(P.ne_ptr + row), ie = __ldg(P.ne_ptr + row + 1);
    // incidences in groups of NG: the group's index loads, then all its
    // element-matrix loads, then the adds in incidence order (the same sums,
    // with NG incidences' memory round trips overlapped instead of one)
    constexpr int NG = LOC == 4 ? 4 : 2;
    for (int q0 = ib; q0 < ie; q0 += NG) {
      int inc[NG];
      uint32_t pw[NG][PW];
#pragma unroll
      for (int u = 0; u < NG; ++u) {
        const bool ok = q0 + u < ie;
        inc[u] = ok ? __ldg(P.ne_col + q0 + u) : 0;
#pragma unroll
        for (int w = 0; w < PW; ++w) pw[u][w] = ok ? __ldg(P.ne_pos + (int64_t)(q0 + u) * PW + w) : 0u;
      }
      double v[NG][LOC], rr[NG];
#pragma unroll
      for (int u = 0; u < NG; ++u) {
        const int e = inc[u] >> 4, a = inc[u] & 15;
        const bool ok = q0 + u < ie;
#pragma unroll
        for (int b = 0; b < LOC; ++b) {
          int k;
          if (SYM) k = a <= b ? a * LOC - (a * (a - 1)) / 2 + (b - a) : b * LOC - (b * (b - 1)) / 2 + (a - b);
          else k = a * LOC + b;
          v[u][b] = ok ? __ldg(P.em + (int64_t)k * E + e) : 0.0;
        }
        rr[u] = ok ? __ldg(P.em + (int64_t)(NK + a) * E + e) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < NG; ++u) {
        if (q0 + u >= ie) break;
#pragma unroll
        for (int b = 0; b < LOC; ++b) {
          const int pos = (pw[u][b >> 2] >> (8 * (b & 3))) & 0xffu;
          if (in_smem) acc[pos * THREADS + t] += v[u][b];
          else P.val[base + pos] += v[u][b];
        }
        r += rr[u];
      }
    }
    if (in_smem)
      for (int k = 0; k < L; ++k) P.val[base + k] = acc[k * THREADS + t];
    P.rhs[row] = r;
  }
}

template <int LOC, bool SYM, int THREADS, int RMAX>
static int launch_pull(const PullArgs& P, cudaStream_t s) {
  const size_t smem = (size_t)RMAX * THREADS * sizeof(double);
  static bool configured = false;
  if (!configured) {
    FL_TRY_CUDA(cudaFuncSetAttribute(k_rows_pull<LOC, SYM, THREADS, RMAX>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured = true;
  }
  // one block per chunk of THREADS consecutive rows, issued in row order: the
  // rows in flight form a contiguous band whose elements' values stay in L2
  const unsigned grid = (unsigned)((P.N + THREADS - 1) / THREADS);
  k_rows_pull<LOC, SYM, THREADS, RMAX><<<grid, THREADS, smem, s>>>(P);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

// Strong Dirichlet (Boundary_Conditions.F90:1983-2025).
__global__ void k_dirichlet(int32_t nb, const int32_t* __restrict__ nodes, int32_t base,
                            const double* __restrict__ gv, const double* __restrict__ t, double dt,
                            int32_t n, double* __restrict__ rhs, uint8_t* __restrict__ inactive,
                            ErrWord* err) {
  note_launch();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nb; k += gridDim.x * blockDim.x) {
    const int i = nodes[k] - base;
    if (i < 0 || i >= n) {
      set_err(err, FL_ERR_ARG, k);
      continue;
    }
    inactive[i] = 1;
    rhs[i] = dt > 0.0 ? (gv[k] - (t ? t[i] : 0.0)) / dt : gv[k];
  }
}

// Row pass with the row-tile index chosen for the mesh: 0, 1, 2 select 64,
// 128, 256 rows per block for P1 (32, 64, 128 for P2).  Shared accumulators
// are sized to the mesh's longest row; longer rows, if any, accumulate in
// place in val.  Every row is summed by one thread in incidence order, so the
// tile changes no result.
template <bool MASS, bool PERM = false>
static int launch_rows_p1_df(const PullArgs& P, int max_row, int tile, cudaStream_t s) {
  if (max_row <= 16) {
    if (tile == 0) return launch_pull_df<64, 16, MASS, PERM>(P, s);
    if (tile == 2) return launch_pull_df<256, 16, MASS, PERM>(P, s);
    return launch_pull_df<128, 16, MASS, PERM>(P, s);
  }
  if (tile == 0) return launch_pull_df<64, 32, MASS, PERM>(P, s);
  if (tile == 2) return launch_pull_df<256, 32, MASS, PERM>(P, s);
  return launch_pull_df<128, 32, MASS, PERM>(P, s);
}

static int launch_rows(const PullArgs& P, int loc, bool use_df, bool closed, int max_row, int tile, cudaStream_t s,
                       bool mass = false) {
  if (loc == 10 && use_df) return launch_rows_p2_hw(P, s);
  if (loc == 4 && use_df)
    return mass ? launch_rows_p1_df<true>(P, max_row, tile, s) : launch_rows_p1_df<false>(P, max_row, tile, s);
  if (loc == 4 && closed) {
    if (tile == 0) return launch_pull<4, true, 64, 32>(P, s);
    if (tile == 2) return launch_pull<4, true, 256, 32>(P, s);
    return launch_pull<4, true, 128, 32>(P, s);
  }
  if (loc == 4) {
    if (tile == 0) return launch_pull<4, false, 64, 32>(P, s);
    if (tile == 2) return launch_pull<4, false, 256, 32>(P, s);
    return launch_pull<4, false, 128, 32>(P, s);
  }
  if (tile == 0) return launch_pull<10, false, 32, 96>(P, s);
  if (tile == 2) return launch_pull<10, false, 128, 96>(P, s);
  return launch_pull<10, false, 64, 96>(P, s);
}

int rows_p1_df(fl_mesh_t* m, const double* em, double* val, double* rhs, cudaStream_t s) {
  FL_CHECK_ARG(m && m->loc == 4 && m->E > 0, "a P1 mesh handle");
  PullArgs P{m->N, m->E, m->ne_ptr.p, m->ne_col.p, nullptr, m->ne_pos.p, m->ndglno.p, m->findrm.p, m->colm.p,
             em, val, rhs, m->err.p, 0, 0};
  return launch_rows_p1_df<false>(P, m->max_row, m->tile_rows == 3 ? 1 : m->tile_rows, s);
}

int rows_p1_closed(fl_mesh_t* m, const double* em, double* val, double* rhs, cudaStream_t s) {
  FL_CHECK_ARG(m && m->loc == 4 && m->E > 0, "a P1 mesh handle");
  PullArgs P{m->N, m->E, m->ne_ptr.p, m->ne_col.p, nullptr, m->ne_pos.p, m->ndglno.p, m->findrm.p, m->colm.p,
             em, val, rhs, m->err.p, 0, 0};
  return launch_rows(P, 4, false, true, m->max_row, m->tile_rows, s);
}

// Per-mesh cache of reference tensors keyed by (field degree, quad degree).
struct TensorCache {
  std::mutex mu;
  struct Entry {
    int device, degree, qdeg;
    RefTensors* d;
  };
  std::vector<Entry> entries;
  const RefTensors* get(int device, int degree, int qdeg, cudaStream_t s) {
    std::lock_guard<std::mutex> lk(mu);
    for (auto& e : entries)
      if (e.device == device && e.degree == degree && e.qdeg == qdeg) return e.d;
    RefTensors h;
    build_tensors(degree, qdeg, h);
    RefTensors* d = nullptr;
    if (cudaMalloc(&d, sizeof(RefTensors)) != cudaSuccess) return nullptr;
    if (cudaMemcpyAsync(d, &h, sizeof(RefTensors), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess) {
      cudaFree(d);
      return nullptr;
    }
    entries.push_back({device, degree, qdeg, d});
    return d;
  }
};
static TensorCache g_tensors;

// Which kernel handles a parameter set: the closed-form P1 kernel covers the
// Poisson/diffusion forms (no advection, no absorption, consistent mass).
static bool diffusion_form(const fl_advdif_params* p) {
  return !p->have_advection && !p->have_absorption && !(p->have_mass && p->lump_mass) && p->have_diffusivity;
}

static bool use_p1_closed_form(const fl_mesh_t* m, const fl_advdif_params* p) {
  return m->loc == 4 && diffusion_form(p);
}

static bool diagonal_kappa(const fl_advdif_params* p) {
  if (p->isotropic_diffusivity) return true;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b)
      if (a != b && p->diffusivity[3 * a + b] != 0.0) return false;
  return true;
}

// The double-float P1 advection-diffusion kernel: P1 field, no absorption,
// a diagonal (or isotropic) kappa, and a symmetric reference mass (every tet
// rule in use; checked).  The pure diffusion forms keep the record kernels.
static bool use_p1_advdif_df(const fl_mesh_t* m, const fl_advdif_params* p, const RefTensors& h) {
  if (m->loc != 4 || diffusion_form(p) || p->have_absorption) return false;
  if (p->have_diffusivity && !diagonal_kappa(p)) return false;
  const double m0 = h.M[0][0], m1 = h.M[0][1];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      const double ref = i == j ? m0 : m1;
      if (fabs(h.M[i][j] - ref) > 1e-14 * fabs(ref)) return false;
    }
  return true;
}

// The double-float P2 kernel: the diffusion form with a diagonal kappa.
static bool use_p2_df(const fl_mesh_t* m, const fl_advdif_params* p) {
  return m->loc == 10 && diffusion_form(p) && diagonal_kappa(p);
}

// Element-record storage per element, in doubles (a double-float pair counts
// as one): P1 closed form 24 (the double-float record is 16 or 24 pairs;
// the FP64 form takes 14 coefficients), P2 double-float 120 (row
// slices of 12 pairs), general forms LOC*(LOC+1) coefficient-major.
size_t assembly_scratch_doubles(const fl_mesh_t* m, const fl_advdif_params* p) {
  const int ncoef = use_p1_closed_form(m, p) ? 24 : use_p2_df(m, p) ? 120 : m->loc * m->loc + m->loc;
  return (size_t)ncoef * m->E;
}

int dirichlet_launch(fl_mesh_t* m, int32_t nb, const int32_t* nodes, int32_t base, const double* g, const double* t,
                     double dt, double* rhs, uint8_t* inactive, cudaStream_t s) {
  if (nb <= 0) return FL_OK;
  k_dirichlet<<<grid_for(nb, 256), 256, 0, s>>>(nb, nodes, base, g, t, dt, m->N, rhs, inactive, m->err.p);
  FL_TRY_CUDA(cudaGetLastError());
  return FL_OK;
}

// Arguments of the P1 double-float element pass (records into em) and its
// term-set key: mass 8, source 4, old field 2, anisotropic kappa 1.
static int p1_df_args(const fl_mesh_t* m, const fl_advdif_params* p, const fl_fields* f, double* em, DfArgs& D) {
  RefTensors h;
  build_tensors(1, p->quad_degree, h);
  const double theta_dt = p->dt * p->theta;
  const bool use_dt = fabs(theta_dt) > 2.220446049250313e-16;
  D = DfArgs{};
  D.E = m->E;
  D.nd = m->ndglno.p;
  D.xnd = m->xndglno.p;
  D.X = m->coords.p;
  D.t = f->t;
  D.f = f->source;
  D.em = reinterpret_cast<float2*>(em);
  const double kap = p->isotropic_diffusivity ? p->diffusivity[0] : 1.0;
  D.kscale = df_host(h.wsum * (use_dt ? theta_dt : 0.0) * kap);
  D.rscale = df_host(h.wsum * kap);
  D.aniso = p->isotropic_diffusivity ? 0 : 1;
  for (int a = 0; a < 3; ++a) D.kdiag[a] = df_host(p->isotropic_diffusivity ? 1.0 : p->diffusivity[4 * a]);
  D.m0 = df_host(h.M[0][0]);
  D.m1 = df_host(h.M[0][1]);
  D.have_mass = p->have_mass;
  D.have_src = p->have_source;
  return (D.have_mass ? 8 : 0) | (D.have_src ? 4 : 0) | (D.t ? 2 : 0) | D.aniso;
}

// Record staging of the P1 double-float element pass: 4.5 or 6.5 kB per warp.
static size_t p1_df_stage_bytes(int threads, int key) {
  return (size_t)(threads / 32) * 32 * ((key & 8) ? 13 : 9) * sizeof(float4);
}

template <bool M, bool S, bool T, bool AN>
static void launch_p1_df_elem(unsigned g, int eb, size_t smem, const DfArgs& D, cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    cudaFuncSetAttribute(k_asm_p1_diffusion_df<M, S, T, AN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)p1_df_stage_bytes(256, M ? 8 : 0));
    configured = true;
  }
  k_asm_p1_diffusion_df<M, S, T, AN><<<g, eb, smem, s>>>(D);
}

static void launch_p1_df_elems(int key, unsigned g, int eb, size_t smem, const DfArgs& D, cudaStream_t s) {
  switch (key) {
#define FL_DF_CASE(K, M, S, T, AN) \
  case K: launch_p1_df_elem<M, S, T, AN>(g, eb, smem, D, s); break;
    FL_DF_CASE(0, false, false, false, false) FL_DF_CASE(1, false, false, false, true)
    FL_DF_CASE(2, false, false, true, false) FL_DF_CASE(3, false, false, true, true)
    FL_DF_CASE(4, false, true, false, false) FL_DF_CASE(5, false, true, false, true)
    FL_DF_CASE(6, false, true, true, false) FL_DF_CASE(7, false, true, true, true)
    FL_DF_CASE(8, true, false, false, false) FL_DF_CASE(9, true, false, false, true)
    FL_DF_CASE(10, true, false, true, false) FL_DF_CASE(11, true, false, true, true)
    FL_DF_CASE(12, true, true, false, false) FL_DF_CASE(13, true, true, false, true)
    FL_DF_CASE(14, true, true, true, false) FL_DF_CASE(15, true, true, true, true)
#undef FL_DF_CASE
  }
}

int assemble(fl_mesh_t* m, const fl_advdif_params* p, const fl_fields* f, double* val, double* rhs,
             cudaStream_t s, double* em_override, bool host_out) {
  FL_CHECK_ARG(m && p && f && val && rhs, "null argument");
  FL_CHECK_ARG(m->E > 0 && (m->loc == 4 || m->loc == 10), "the handle has no elements (pattern-only handle)");
  FL_CHECK_ARG(p->quad_degree >= 1 && p->quad_degree <= 4, "quadrature degree 1..4");
  FL_CHECK_ARG(!p->have_advection || f->velocity, "advection needs a velocity field");
  FL_CHECK_ARG(!p->have_source || f->source, "source field missing");
  FL_CHECK_ARG(!p->have_absorption || f->absorption, "absorption field missing");
  const int degree = m->loc == 4 ? 1 : 2;
  const RefTensors* ref = g_tensors.get(m->device, degree, p->quad_degree, s);
  if (!ref) {
    set_error("reference tensor upload failed");
    return FL_ERR_CUDA;
  }
  // zero(matrix); zero(rhs) (Advection_Diffusion_CG.F90:560-561) happen in the
  // row pass, which writes every entry of val and rhs.
  AsmArgs A{};
  A.E = m->E;
  A.nd = m->ndglno.p;
  A.xnd = m->xndglno.p;
  A.X = m->coords.p;
  A.t = f->t;
  A.u = f->velocity;
  A.f = f->source;
  A.alpha = f->absorption;
  A.ref = ref;
  A.theta_dt = p->dt * p->theta;
  // epsilon(0.0) is the real(8) machine epsilon under -fdefault-real-8
  const double eps = 2.220446049250313e-16;
  A.use_dt = fabs(A.theta_dt) > eps;
  // the divergence coefficient: beta, or -(1 - beta) by parts (applied when
  // |beta| resp. |1 - beta| exceeds epsilon, :1037 and :1087)
  A.by_parts = p->integrate_advection_by_parts != 0;
  A.beta = A.by_parts ? -(1.0 - p->beta) : p->beta;
  A.have_beta = p->have_advection && fabs(A.by_parts ? 1.0 - p->beta : p->beta) > eps;
  for (int k = 0; k < 9; ++k) A.kappa[k] = p->diffusivity[k];
  A.have_mass = p->have_mass;
  A.lump = p->have_mass && p->lump_mass;
  A.have_adv = p->have_advection;
  A.have_diff = p->have_diffusivity;
  A.iso = p->isotropic_diffusivity;
  A.have_src = p->have_source;
  A.have_abs = p->have_absorption;
  const bool closed = use_p1_closed_form(m, p);
  const bool p2df = use_p2_df(m, p);
  RefTensors h1;
  bool p1adv = false;
  if (m->loc == 4 && !diffusion_form(p) && !p->have_absorption) {
    build_tensors(1, p->quad_degree, h1);
    p1adv = use_p1_advdif_df(m, p, h1);
  }
  const int loc = m->loc;
  double* em = em_override;
  if (!em) {
    FL_TRY(m->em.reserve(assembly_scratch_doubles(m, p)));
    em = m->em.p;
  }
  A.em = em;
  // element-pass tiles (the autotuner's choice; results do not depend on it)
  const int eb = m->tile_elem_block, esm = m->tile_elem_per_sm;
  if (m->timing) {
    if (!m->ev0) {
      FL_TRY_CUDA(cudaEventCreate(&m->ev0));
      FL_TRY_CUDA(cudaEventCreate(&m->ev1));
    }
    FL_TRY_CUDA(cudaEventRecord(m->ev0, s));
  }
  // Diagonal (or isotropic) kappa: the double-float element passes; a full
  // tensor keeps the FP64 forms.
  const bool use_df = (closed && diagonal_kappa(p)) || p2df;
  if (p2df) {
    RefTensors h;
    build_tensors(2, p->quad_degree, h);
    DfP2Args D{};
    D.E = m->E;
    D.nd = m->ndglno.p;
    D.xnd = m->xndglno.p;
    D.X = m->coords.p;
    D.t = f->t;
    D.f = f->source;
    D.em = reinterpret_cast<float4*>(em);
    for (int i = 0; i < 10; ++i)
      for (int j = i; j < 10; ++j) {
        const int q = sym10(i, j);
        const double (*R)[3] = h.R[i][j];
        D.S[q][0] = df_host(R[0][0]);
        D.S[q][1] = df_host(R[1][1]);
        D.S[q][2] = df_host(R[2][2]);
        D.S[q][3] = df_host(R[0][1] + R[1][0]);
        D.S[q][4] = df_host(R[0][2] + R[2][0]);
        D.S[q][5] = df_host(R[1][2] + R[2][1]);
        D.M[q] = df_host(h.M[i][j]);
      }
    D.qs = df_host(A.use_dt ? A.theta_dt : 0.0);
    for (int a = 0; a < 3; ++a)
      D.kdiag[a] = df_host(p->isotropic_diffusivity ? p->diffusivity[0] : p->diffusivity[4 * a]);
    D.have_mass = p->have_mass;
    D.have_src = p->have_source;
    const size_t dsmem = (size_t)45 * kP2Threads * sizeof(float2);
    static bool p2_configured = false;
    if (!p2_configured) {
      FL_TRY_CUDA(cudaFuncSetAttribute(k_asm_p2_diffusion_df, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)dsmem));
      p2_configured = true;
    }
    k_asm_p2_diffusion_df<<<grid_for(m->E, kP2Threads, esm), kP2Threads, dsmem, s>>>(D);
  } else if (use_df) {
    DfArgs D{};
    const int key = p1_df_args(m, p, f, em, D);
    const unsigned g = grid_for(m->E, eb, esm);
    const size_t smem = p1_df_stage_bytes(eb, key);
    if (m->tile_rows == 3 && !em_override) {
      // fused element + row pass (same sums, records kept in L2)
      FL_TRY(fused_plan(m, s));
      if (m->fz_state == 1) {
        PullArgs P{m->N, m->E, m->ne_ptr.p, m->ne_col.p, m->fz_rec.p, m->ne_pos.p, m->ndglno.p, m->findrm.p,
                   m->colm.p, em, val, rhs, m->err.p, host_out ? 1 : 0, 0};
        switch (key) {
#define FL_FZ_CASE(K, M, S, T, AN) \
  case K: FL_TRY((launch_fused<M, S, T, AN>(m, D, P, s))); break;
          FL_FZ_CASE(0, false, false, false, false) FL_FZ_CASE(1, false, false, false, true)
          FL_FZ_CASE(2, false, false, true, false) FL_FZ_CASE(3, false, false, true, true)
          FL_FZ_CASE(4, false, true, false, false) FL_FZ_CASE(5, false, true, false, true)
          FL_FZ_CASE(6, false, true, true, false) FL_FZ_CASE(7, false, true, true, true)
          FL_FZ_CASE(8, true, false, false, false) FL_FZ_CASE(9, true, false, false, true)
          FL_FZ_CASE(10, true, false, true, false) FL_FZ_CASE(11, true, false, true, true)
          FL_FZ_CASE(12, true, true, false, false) FL_FZ_CASE(13, true, true, false, true)
          FL_FZ_CASE(14, true, true, true, false) FL_FZ_CASE(15, true, true, true, true)
#undef FL_FZ_CASE
        }
        if (m->timing) {
          FL_TRY_CUDA(cudaEventRecord(m->ev1, s));
          m->timed = true;
        }
        return FL_OK;
      }
    }
    launch_p1_df_elems(key, g, eb, smem, D, s);
  } else if (closed) {
    k_asm_p1_diffusion<<<grid_for(m->E, eb, esm), eb, 0, s>>>(A);
  } else if (p1adv) {
    AdvDfArgs D{};
    D.E = m->E;
    D.nd = m->ndglno.p;
    D.xnd = m->xndglno.p;
    D.X = m->coords.p;
    D.t = f->t;
    D.u = f->velocity;
    D.f = f->source;
    D.em = em;
    D.m0 = df_host(h1.M[0][0]);
    D.m1 = df_host(h1.M[0][1]);
    D.dm = df_host(h1.M[0][0] - h1.M[0][1]);
    D.ml = df_host(h1.M[0][0] + 3.0 * h1.M[0][1]);
    for (int a = 0; a < 3; ++a)
      D.kd[a] = df_host(h1.wsum * (p->isotropic_diffusivity ? p->diffusivity[0] : p->diffusivity[4 * a]));
    D.qs = df_host(A.use_dt ? A.theta_dt : 0.0);
    D.beta = df_host(A.beta);
    D.have_mass = A.have_mass;
    D.lump = A.lump;
    D.by_parts = A.by_parts;
    D.have_beta = A.have_beta;
    D.have_diff = A.have_diff;
    D.have_src = A.have_src;
    if (A.have_adv) k_asm_p1_advdif_df<true><<<grid_for(m->E, 128, esm), 128, 0, s>>>(D);
    else k_asm_p1_advdif_df<false><<<grid_for(m->E, 128, esm), 128, 0, s>>>(D);
  } else if (loc == 4) {
    k_asm_general<4><<<grid_for(m->E, 128, esm), 128, 0, s>>>(A);
  } else {
    k_asm_general<10><<<grid_for(m->E, 128, esm), 128, 0, s>>>(A);
  }
  FL_TRY_CUDA(cudaGetLastError());
  PullArgs P{m->N, m->E, m->ne_ptr.p, m->ne_col.p, nullptr, m->ne_pos.p, m->ndglno.p, m->findrm.p, m->colm.p,
             em, val, rhs, m->err.p, host_out ? 1 : 0, 0};
  FL_TRY(launch_rows(P, loc, use_df, closed, m->max_row, m->tile_rows, s, p->have_mass != 0));
  if (m->timing) {
    FL_TRY_CUDA(cudaEventRecord(m->ev1, s));
    m->timed = true;
  }
  return FL_OK;
}

// Pinned host outputs of the P1 double-float forms: the assembly runs in the
// row chunks of the fused plan on three streams.  The copy stream uploads
// each chunk's field values and takes each finished chunk's val and rhs
// ranges back; the element pass of chunk k+1 (stream s) runs beside the row
// pass of chunk k (the row stream).  The host link, the bound of this call,
// so starts after the first (small) chunk instead of after the whole
// assembly.  Element records sit in the fused plan's order and the row pass
// reads them through its slice map, summing every row in the same order as
// the device path: val and rhs are bit-identical to it.  *done stays false
// (nothing enqueued) when the mesh or the form does not take this path.  The
// caller synchronises the copy and row streams before the host arrays are
// used.
static int assemble_pipelined(fl_mesh_t* m, const fl_advdif_params* p, const fl_fields* hf, double* hval,
                              double* hrhs, cudaStream_t s, bool* done) {
  *done = false;
  if (!(use_p1_closed_form(m, p) && diagonal_kappa(p))) return FL_OK;
  if (m->nnz * (int64_t)sizeof(double) / kCkBytes < 2) return FL_OK;  // fewer than two chunks
  FL_CHECK_ARG(!p->have_source || hf->source, "source field missing");
  FL_TRY(fused_plan(m, s));
  const int K = (int)m->ck_rows.size() - 1;
  if (m->fz_state != 1 || K < 2) return FL_OK;
  FL_TRY(m->em.reserve(assembly_scratch_doubles(m, p)));
  FL_TRY(m->st_val.reserve(m->nnz));
  FL_TRY(m->st_rhs.reserve(m->N));
  for (cudaStream_t& q : m->ck_streams)
    if (!q) FL_TRY_CUDA(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking));
  // events: [k] rows of chunk k written, [K+k] its fields uploaded, [2K+k]
  // its element records written, [3K] the call's start, [3K+1] all rows
  while ((int)m->ck_ev.size() < 3 * K + 2) {
    cudaEvent_t e = nullptr;
    FL_TRY_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    m->ck_ev.push_back(e);
  }
  cudaEvent_t* ev = m->ck_ev.data();
  const cudaStream_t cs = m->ck_streams[0], rs = m->ck_streams[1];
  // the copy and row streams follow the work already on s (earlier calls'
  // use of the staging buffers and records)
  FL_TRY_CUDA(cudaEventRecord(ev[3 * K], s));
  for (cudaStream_t q : m->ck_streams) FL_TRY_CUDA(cudaStreamWaitEvent(q, ev[3 * K], 0));
  fl_fields f{nullptr, nullptr, nullptr, nullptr};
  const double* src = p->have_source ? hf->source : nullptr;
  if (src) FL_TRY(m->st_src.reserve(m->N));
  if (hf->t) FL_TRY(m->st_t.reserve(m->N));
  f.source = src ? m->st_src.p : nullptr;
  f.t = hf->t ? m->st_t.p : nullptr;
  for (int k = 0; k < K; ++k) {
    const int32_t a = m->ck_node[k], b = m->ck_node[k + 1];
    if (b > a) {
      if (src)
        FL_TRY_CUDA(cudaMemcpyAsync(m->st_src.p + a, src + a, sizeof(double) * (size_t)(b - a),
                                    cudaMemcpyHostToDevice, cs));
      if (hf->t)
        FL_TRY_CUDA(cudaMemcpyAsync(m->st_t.p + a, hf->t + a, sizeof(double) * (size_t)(b - a),
                                    cudaMemcpyHostToDevice, cs));
    }
    FL_TRY_CUDA(cudaEventRecord(ev[K + k], cs));
  }
  DfArgs D{};
  const int key = p1_df_args(m, p, &f, m->em.p, D);
  D.perm = m->fz_perm.p;
  const int eb = m->tile_elem_block, esm = m->tile_elem_per_sm;
  const int tile = m->tile_rows == 3 ? 1 : m->tile_rows;
  const size_t smem = p1_df_stage_bytes(eb, key);
  PullArgs P{m->N, m->E, m->ne_ptr.p, m->ne_col.p, m->fz_rec.p, m->ne_pos.p, m->ndglno.p, m->findrm.p,
             m->colm.p, m->em.p, m->st_val.p, m->st_rhs.p, m->err.p, 0, 0};
  if (m->timing) {
    if (!m->ev0) {
      FL_TRY_CUDA(cudaEventCreate(&m->ev0));
      FL_TRY_CUDA(cudaEventCreate(&m->ev1));
    }
    FL_TRY_CUDA(cudaEventRecord(m->ev0, s));
  }
  for (int k = 0; k < K; ++k) {
    D.p0 = m->ck_elem[k];
    D.E = m->ck_elem[k + 1];
    FL_TRY_CUDA(cudaStreamWaitEvent(s, ev[K + k], 0));
    if (D.E > D.p0) launch_p1_df_elems(key, grid_for(D.E - D.p0, eb, esm), eb, smem, D, s);
    FL_TRY_CUDA(cudaGetLastError());
    FL_TRY_CUDA(cudaEventRecord(ev[2 * K + k], s));
    FL_TRY_CUDA(cudaStreamWaitEvent(rs, ev[2 * K + k], 0));
    P.row0 = m->ck_rows[k];
    P.N = m->ck_rows[k + 1];
    if (p->have_mass) {
      FL_TRY((launch_rows_p1_df<true, true>(P, m->max_row, tile, rs)));
    } else {
      FL_TRY((launch_rows_p1_df<false, true>(P, m->max_row, tile, rs)));
    }
    FL_TRY_CUDA(cudaEventRecord(ev[k], rs));
    FL_TRY_CUDA(cudaStreamWaitEvent(cs, ev[k], 0));
    const int64_t v0 = m->ck_val[k], v1 = m->ck_val[k + 1];
    if (v1 > v0)
      FL_TRY_CUDA(cudaMemcpyAsync(hval + v0, m->st_val.p + v0, sizeof(double) * (size_t)(v1 - v0),
                                  cudaMemcpyDeviceToHost, cs));
    FL_TRY_CUDA(cudaMemcpyAsync(hrhs + P.row0, m->st_rhs.p + P.row0, sizeof(double) * (size_t)(P.N - P.row0),
                                cudaMemcpyDeviceToHost, cs));
  }
  // s (error word, timing, the next call) follows the row stream
  FL_TRY_CUDA(cudaEventRecord(ev[3 * K + 1], rs));
  FL_TRY_CUDA(cudaStreamWaitEvent(s, ev[3 * K + 1], 0));
  if (m->timing) {
    FL_TRY_CUDA(cudaEventRecord(m->ev1, s));
    m->timed = true;
  }
  *done = true;
  return FL_OK;
}

// Tile autotuner: times the assembly of this mesh and parameter set under
// each element-pass tile (threads per block x blocks per SM) and then each
// row-pass tile, keeping the fastest of each (median of three timed runs
// after one warm-up).  The candidates only regroup independent elements and
// rows, so val and rhs are the same under every choice; they hold the
// assembled system on return.
int autotune_assembly(fl_mesh_t* m, const fl_advdif_params* p, const fl_fields* f, double* val, double* rhs,
                      cudaStream_t s) {
  static const int kBlocks[] = {128, 256};
  static const int kPerSm[] = {4, 8, 16, 32};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  FL_TRY_CUDA(cudaEventCreate(&e0));
  FL_TRY_CUDA(cudaEventCreate(&e1));
  const bool timing = m->timing;
  m->timing = false;
  auto time_one = [&](float* ms) -> int {
    float t[3];
    FL_TRY(assemble(m, p, f, val, rhs, s, nullptr));
    for (int k = 0; k < 3; ++k) {
      FL_TRY_CUDA(cudaEventRecord(e0, s));
      FL_TRY(assemble(m, p, f, val, rhs, s, nullptr));
      FL_TRY_CUDA(cudaEventRecord(e1, s));
      FL_TRY_CUDA(cudaEventSynchronize(e1));
      FL_TRY_CUDA(cudaEventElapsedTime(&t[k], e0, e1));
    }
    std::sort(t, t + 3);
    *ms = t[1];
    return FL_OK;
  };
  int st = FL_OK;
  do {
    float best = 1e30f;
    int bb = m->tile_elem_block, bs = m->tile_elem_per_sm;
    for (int b : kBlocks)
      for (int ps : kPerSm) {
        m->tile_elem_block = b;
        m->tile_elem_per_sm = ps;
        float ms = 0.f;
        if ((st = time_one(&ms)) != FL_OK) break;
        if (ms < best) {
          best = ms;
          bb = b;
          bs = ps;
        }
      }
    m->tile_elem_block = bb;
    m->tile_elem_per_sm = bs;
    if (st != FL_OK) break;
    best = 1e30f;
    int br = m->tile_rows;
    const int nrt = (use_p1_closed_form(m, p) && diagonal_kappa(p)) ? 4 : 3;  // 3: fused P1 pass
    for (int r = 0; r < nrt; ++r) {
      m->tile_rows = r;
      float ms = 0.f;
      if ((st = time_one(&ms)) != FL_OK) break;
      if (ms < best) {
        best = ms;
        br = r;
      }
    }
    m->tile_rows = br;
    if (st != FL_OK) break;
    st = assemble(m, p, f, val, rhs, s, nullptr);
    m->tuned = true;
  } while (0);
  m->timing = timing;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return st;
}

}  // namespace fl

using namespace fl;

static cudaStream_t pick_stream(fl_mesh m, void* stream) {
  return stream ? (cudaStream_t)stream : m->stream;
}

extern "C" int fl_dev_assemble_advdif_cg(fl_mesh m, const fl_advdif_params* p, const fl_fields* f,
                                         double* val, double* rhs, void* stream) {
  FL_CHECK_ARG(m, "null mesh");
  cudaStream_t s = pick_stream(m, stream);
  FL_TRY(assemble(m, p, f, val, rhs, s, nullptr));
  // pattern misses are reported synchronously, as FLAbort is in the reference
  return check_err(m->err.p, s, "Attempting to set value in matrix outside sparsity pattern");
}

// Device view of a host array that is page-locked and mapped (cudaHostAlloc,
// cudaHostRegister, or a pinned buffer of the caller's allocator); null for
// pageable memory.
static double* mapped_host(double* h) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? static_cast<double*>(a.devicePointer) : nullptr;
}

extern "C" int fl_gpu_assemble_advdif_cg(fl_mesh m, const fl_advdif_params* p, const fl_fields* f,
                                         double* val, double* rhs) {
  FL_CHECK_ARG(m && p && f && val && rhs, "null argument");
  cudaStream_t s = m->stream;
  // Pinned output arrays: the row pass writes val and rhs into host memory
  // itself (each entry once), so the transfer overlaps the row pass instead
  // of following it.  Pageable arrays go through device staging buffers.
  double* mval = mapped_host(val);
  double* mrhs = mval ? mapped_host(rhs) : nullptr;
  if (mrhs) {
    // P1 double-float forms: chunked uploads, assembly and copies back
    bool done = false;
    int st = assemble_pipelined(m, p, f, val, rhs, s, &done);
    if (st == FL_OK && done) st = check_err(m->err.p, s, "Attempting to set value in matrix outside sparsity pattern");
    // row passes and copies still in flight (also after an error) end
    // before the caller's arrays are touched
    for (cudaStream_t q : m->ck_streams) {
      if (!q) continue;
      const cudaError_t e = cudaStreamSynchronize(q);
      if (st == FL_OK && e != cudaSuccess) {
        set_error("pipelined assembly: %s", cudaGetErrorString(e));
        st = FL_ERR_CUDA;
      }
    }
    if (st != FL_OK || done) return st;
  } else {
    FL_TRY(m->st_val.reserve(m->nnz));
    FL_TRY(m->st_rhs.reserve(m->N));
  }
  fl_fields df{nullptr, nullptr, nullptr, nullptr};
  auto up = [&](const double* h, DevBuf<double>& d, size_t n, const double** out) -> int {
    if (!h) return FL_OK;
    FL_TRY(d.reserve(n));
    FL_TRY_CUDA(cudaMemcpyAsync(d.p, h, sizeof(double) * n, cudaMemcpyHostToDevice, s));
    *out = d.p;
    return FL_OK;
  };
  FL_TRY(up(f->t, m->st_t, m->N, &df.t));
  FL_TRY(up(p->have_advection ? f->velocity : nullptr, m->st_u, (size_t)3 * m->Nx, &df.velocity));
  FL_TRY(up(p->have_source ? f->source : nullptr, m->st_src, m->N, &df.source));
  FL_TRY(up(p->have_absorption ? f->absorption : nullptr, m->st_abs, m->N, &df.absorption));
  if (mrhs) {
    FL_TRY(assemble(m, p, &df, mval, mrhs, s, nullptr, true));
    return check_err(m->err.p, s, "Attempting to set value in matrix outside sparsity pattern");
  }
  FL_TRY(fl_dev_assemble_advdif_cg(m, p, &df, m->st_val.p, m->st_rhs.p, s));
  FL_TRY_CUDA(cudaMemcpyAsync(val, m->st_val.p, sizeof(double) * m->nnz, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaMemcpyAsync(rhs, m->st_rhs.p, sizeof(double) * m->N, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  return FL_OK;
}

extern "C" int fl_dev_autotune_assembly(fl_mesh m, const fl_advdif_params* p, const fl_fields* f, double* val,
                                        double* rhs, void* stream, int32_t* tiles) {
  FL_CHECK_ARG(m && p && f && val && rhs, "null argument");
  cudaStream_t s = pick_stream(m, stream);
  FL_TRY(autotune_assembly(m, p, f, val, rhs, s));
  if (tiles) {
    tiles[0] = m->tile_elem_block;
    tiles[1] = m->tile_elem_per_sm;
    tiles[2] = m->tile_rows;
  }
  return check_err(m->err.p, s, "Attempting to set value in matrix outside sparsity pattern");
}

extern "C" int fl_set_assembly_tiles(fl_mesh m, int32_t elem_block, int32_t elem_blocks_per_sm, int32_t row_tile) {
  FL_CHECK_ARG(m, "null mesh");
  FL_CHECK_ARG(elem_block == 128 || elem_block == 256, "element block 128 or 256");
  FL_CHECK_ARG(elem_blocks_per_sm >= 1 && elem_blocks_per_sm <= 64, "element blocks per SM 1..64");
  FL_CHECK_ARG(row_tile >= 0 && row_tile <= 3, "row tile 0..3 (3: fused P1 element and row pass)");
  m->tile_elem_block = elem_block;
  m->tile_elem_per_sm = elem_blocks_per_sm;
  m->tile_rows = row_tile;
  return FL_OK;
}

extern "C" int fl_get_assembly_tiles(fl_mesh m, int32_t* tiles) {
  FL_CHECK_ARG(m && tiles, "null argument");
  tiles[0] = m->tile_elem_block;
  tiles[1] = m->tile_elem_per_sm;
  tiles[2] = m->tile_rows;
  return FL_OK;
}

extern "C" int fl_set_kernel_timing(fl_mesh m, int32_t on) {
  FL_CHECK_ARG(m, "null mesh");
  m->timing = on != 0;
  m->timed = false;
  return FL_OK;
}

extern "C" int fl_last_assembly_kernel_ms(fl_mesh m, float* ms) {
  FL_CHECK_ARG(m && ms, "null argument");
  FL_CHECK_ARG(m->timed, "no timed assembly recorded (enable fl_set_kernel_timing first)");
  FL_TRY_CUDA(cudaEventSynchronize(m->ev1));
  FL_TRY_CUDA(cudaEventElapsedTime(ms, m->ev0, m->ev1));
  return FL_OK;
}

namespace fl {

// ------------------------------------------------- allocation-free variant --
// Some callers cannot allocate device memory at the point where they assemble:
// a host application whose memory manager has reserved the device's memory
// up front, or a time-stepping loop that must not call cudaMalloc (which can
// synchronise the whole device).  For them, the P1 diffusion assembly (the
// pressure-Poisson form) runs with its element-matrix scratch in a fixed,
// file-scope device array instead of the handle's grow-only buffer.
//
// Limit: meshes of at most kNoAllocMaxElements elements (14 doubles of scratch
// per element, 14.7 MB held by every GPU that loads the library until exit).
// The array is shared by every call: the element pass writes every value the
// row pass reads, so nothing needs clearing between calls, but calls whose
// work overlaps on the GPU (different streams or threads) race on it.
constexpr int kNoAllocMaxElements = 131072;
constexpr int kNoAllocCoef = 14;  // 10 symmetric matrix entries + 4 rhs entries
static __device__ __align__(256) double g_noalloc_em[(size_t)kNoAllocCoef * kNoAllocMaxElements];
static __device__ __align__(256) RefTensors g_noalloc_ref[4];  // quadrature degrees 1..4

// Host-side device addresses of the arrays above, resolved once per device by
// cudaGetSymbolAddress (the array's name in host code is not a device address).
// They belong to the device's current context: cudaDeviceReset discards them
// (and the uploaded tables) together with every mesh handle, so a process that
// resets a device must unload and reload the library before calling again.
struct NoAllocDevice {
  bool ready = false;
  double* em = nullptr;
  RefTensors* ref = nullptr;
};
static std::mutex g_noalloc_mu;
static NoAllocDevice g_noalloc_dev[64];

static int noalloc_setup(int dev, NoAllocDevice** out) {
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  FL_CHECK_ARG(dev >= 0 && dev < 64, "device ordinal");
  NoAllocDevice& d = g_noalloc_dev[dev];
  if (!d.ready) {
    void* p = nullptr;
    FL_TRY_CUDA(cudaGetSymbolAddress(&p, g_noalloc_em));
    d.em = static_cast<double*>(p);
    FL_TRY_CUDA(cudaGetSymbolAddress(&p, g_noalloc_ref));
    d.ref = static_cast<RefTensors*>(p);
    for (int q = 1; q <= 4; ++q) {
      RefTensors h;
      build_tensors(1, q, h);
      FL_TRY_CUDA(cudaMemcpyToSymbol(g_noalloc_ref, &h, sizeof(RefTensors), sizeof(RefTensors) * (q - 1),
                                     cudaMemcpyHostToDevice));
    }
    // cudaMemcpyToSymbol from pageable memory may return before the data has
    // reached the device, and it is ordered on the legacy default stream only:
    // the assembly's stream (often non-blocking) must not start before the
    // tables are complete.  This runs once per device.
    FL_TRY_CUDA(cudaDeviceSynchronize());
    d.ready = true;
  }
  *out = &d;
  return FL_OK;
}

}  // namespace fl

extern "C" int fl_dev_assemble_p1_diffusion_noalloc(fl_mesh m, const fl_advdif_params* p, const fl_fields* f,
                                                    double* val, double* rhs, void* stream) {
  using namespace fl;
  FL_CHECK_ARG(m && p && f && val && rhs, "null argument");
  FL_CHECK_ARG(m->loc == 4, "allocation-free assembly supports P1 field meshes only");
  FL_CHECK_ARG(use_p1_closed_form(m, p), "allocation-free assembly supports the diffusion form only "
               "(diffusivity, optional source and consistent mass; no advection or absorption)");
  FL_CHECK_ARG(p->quad_degree >= 1 && p->quad_degree <= 4, "quadrature degree 1..4");
  FL_CHECK_ARG(!p->have_source || f->source, "source field missing");
  if (m->E > kNoAllocMaxElements) {
    set_error("invalid argument: %d elements exceed the allocation-free limit of %d", m->E,
              kNoAllocMaxElements);
    return FL_ERR_ARG;
  }
  int dev = 0;
  FL_TRY_CUDA(cudaGetDevice(&dev));
  NoAllocDevice* d = nullptr;
  FL_TRY(noalloc_setup(dev, &d));
  cudaStream_t s = stream ? (cudaStream_t)stream : m->stream;
  AsmArgs A{};
  A.E = m->E;
  A.nd = m->ndglno.p;
  A.xnd = m->xndglno.p;
  A.X = m->coords.p;
  A.t = f->t;
  A.f = f->source;
  A.em = d->em;
  A.ref = d->ref + (p->quad_degree - 1);
  A.theta_dt = p->dt * p->theta;
  const double eps = 2.220446049250313e-16;
  A.use_dt = fabs(A.theta_dt) > eps;
  for (int k = 0; k < 9; ++k) A.kappa[k] = p->diffusivity[k];
  A.have_mass = p->have_mass;
  A.have_diff = p->have_diffusivity;
  A.iso = p->isotropic_diffusivity;
  A.have_src = p->have_source;
  k_asm_p1_diffusion<<<grid_for(m->E, 256, 16), 256, 0, s>>>(A);
  FL_TRY_CUDA(cudaGetLastError());
  PullArgs P{m->N, m->E, m->ne_ptr.p, m->ne_col.p, nullptr, m->ne_pos.p, m->ndglno.p, m->findrm.p, m->colm.p,
             d->em, val, rhs, m->err.p, 0, 0};
  FL_TRY((launch_pull<4, true, 128, 32>(P, s)));
  return check_err(m->err.p, s, "Attempting to set value in matrix outside sparsity pattern");
}

extern "C" int fl_dev_apply_dirichlet(fl_mesh m, int32_t nb, const int32_t* nodes, int32_t base,
                                      const double* g, const double* t, double dt, double* rhs,
                                      uint8_t* inactive, void* stream) {
  FL_CHECK_ARG(m && rhs && inactive, "null argument");
  FL_CHECK_ARG(nb >= 0 && (nb == 0 || (nodes && g)), "boundary node list");
  if (nb == 0) return FL_OK;
  cudaStream_t s = pick_stream(m, stream);
  k_dirichlet<<<grid_for(nb, 256), 256, 0, s>>>(nb, nodes, base, g, t, dt, m->N, rhs, inactive, m->err.p);
  FL_TRY_CUDA(cudaGetLastError());
  return check_err(m->err.p, s, "Dirichlet node out of range");
}

extern "C" int fl_gpu_apply_dirichlet(fl_mesh m, int32_t nb, const int32_t* nodes, int32_t base,
                                      const double* g, const double* t, double dt, double* rhs,
                                      uint8_t* inactive) {
  FL_CHECK_ARG(m && rhs && inactive, "null argument");
  FL_CHECK_ARG(nb >= 0 && (nb == 0 || (nodes && g)), "boundary node list");
  cudaStream_t s = m->stream;
  FL_TRY(m->st_rhs.reserve(m->N));
  FL_TRY(m->st_ina.reserve(m->N));
  FL_TRY_CUDA(cudaMemcpyAsync(m->st_rhs.p, rhs, sizeof(double) * m->N, cudaMemcpyHostToDevice, s));
  FL_TRY_CUDA(cudaMemcpyAsync(m->st_ina.p, inactive, m->N, cudaMemcpyHostToDevice, s));
  if (nb > 0) {
    FL_TRY(m->st_nodes.reserve(nb));
    FL_TRY(m->st_g.reserve(nb));
    FL_TRY_CUDA(cudaMemcpyAsync(m->st_nodes.p, nodes, sizeof(int32_t) * nb, cudaMemcpyHostToDevice, s));
    FL_TRY_CUDA(cudaMemcpyAsync(m->st_g.p, g, sizeof(double) * nb, cudaMemcpyHostToDevice, s));
  }
  const double* tp = nullptr;
  if (t) {
    FL_TRY(m->st_t.reserve(m->N));
    FL_TRY_CUDA(cudaMemcpyAsync(m->st_t.p, t, sizeof(double) * m->N, cudaMemcpyHostToDevice, s));
    tp = m->st_t.p;
  }
  FL_TRY(fl_dev_apply_dirichlet(m, nb, m->st_nodes.p, base, m->st_g.p, tp, dt, m->st_rhs.p, m->st_ina.p, s));
  FL_TRY_CUDA(cudaMemcpyAsync(rhs, m->st_rhs.p, sizeof(double) * m->N, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaMemcpyAsync(inactive, m->st_ina.p, m->N, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  return FL_OK;
}

// ------------------------------------------------------------ surface loop --
// assemble_advection_diffusion_face_cg (Advection_Diffusion_CG.F90:1228-1286)
// for every surface element, added row by row: one thread per field node adds
// the faces holding it in ascending face order (the reference's face loop
// order), so the sums are deterministic.  Faces are O(n^2) against O(n^3)
// elements, so the face quantities are simply recomputed for each of a face's
// nodes, in FP64.
namespace fl {

struct FaceAsmArgs {
  int32_t N, floc, base, E;
  const int32_t* fptr;
  const int32_t* flist;
  const int32_t* faces;
  const int32_t* xfaces;
  const int32_t* face_ele;
  const int32_t* bc_type;
  const double* bc1;
  const double* bc2;
  const int32_t* xnd;
  const double* X;
  const double* u;   // P1 velocity on the coordinate mesh (3 per vertex)
  const double* t;
  const int32_t* findrm;
  const int32_t* colm;
  double* val;
  double* rhs;
  double theta, dt_theta;
  int adv, diff, use_dt, ngi;
  double ql[6][3];  // barycentric coordinates of the triangle rule's points
  double qw[6];
  ErrWord* err;
};

// Lagrange functions of the face (P1: barycentrics; P2: vertex L(2L-1),
// edge 4 L_a L_b, in the triangle's local order).
__device__ __forceinline__ void face_shape(int floc, const double l[3], double* n) {
  if (floc == 3) {
    n[0] = l[0];
    n[1] = l[1];
    n[2] = l[2];
    return;
  }
  n[0] = l[0] * (2.0 * l[0] - 1.0);
  n[1] = (2.0 * l[0]) * (2.0 * l[1]);
  n[2] = l[1] * (2.0 * l[1] - 1.0);
  n[3] = (2.0 * l[0]) * (2.0 * l[2]);
  n[4] = (2.0 * l[1]) * (2.0 * l[2]);
  n[5] = l[2] * (2.0 * l[2] - 1.0);
}

__global__ void __launch_bounds__(128) k_advdif_faces(FaceAsmArgs F) {
  note_launch();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < F.N; i += gridDim.x * blockDim.x) {
    const int qb = F.fptr[i], qe = F.fptr[i + 1];
    for (int q = qb; q < qe; ++q) {
      const int f = F.flist[q];
      const int ty = F.bc_type ? F.bc_type[f] : 0;
      if (ty == 3) continue;  // internal
      if (ty != 0 && ty != 1 && ty != 2 && ty != 4) {
        set_err(F.err, FL_ERR_ARG, f);
        continue;
      }
      if (ty == 2 && F.diff) {  // FLExit in add_diffusivity_face_cg
        set_err(F.err, FL_ERR_ARG, f);
        continue;
      }
      const bool dface = F.diff && (ty == 1 || ty == 4);
      if (!F.adv && !dface) continue;
      // the values a face needs: t_bc for neumann, robin and (advected) weak
      // Dirichlet faces, t_bc_2 for robin faces
      if (((dface || (F.adv && ty == 2)) && !F.bc1) || (dface && ty == 4 && !F.bc2)) {
        set_err(F.err, FL_ERR_ARG, f);
        continue;
      }
      const int floc = F.floc;
      int fn[6], li = -1;
      for (int j = 0; j < floc; ++j) {
        fn[j] = F.faces[(int64_t)floc * f + j] - F.base;
        if (fn[j] == i) li = j;
      }
      int xv[3];
      for (int j = 0; j < 3; ++j) xv[j] = F.xfaces[3 * (int64_t)f + j] - F.base;
      if (li < 0) {
        set_err(F.err, FL_ERR_ARG, f);
        continue;
      }
      double Xf[3][3];
      for (int j = 0; j < 3; ++j)
        for (int a = 0; a < 3; ++a) Xf[j][a] = F.X[3 * (int64_t)xv[j] + a];
      // transform_facet_to_physical: J = [X1 - X3, X2 - X3], detJ = |J1 x J2|
      double J[3][2];
      for (int a = 0; a < 3; ++a) {
        J[a][0] = Xf[0][a] - Xf[2][a];
        J[a][1] = Xf[1][a] - Xf[2][a];
      }
      double detJ = 0.0;
      for (int k = 1; k <= 3; ++k) {
        const int c2 = (k + 1) % 3, c1 = k % 3;
        const double v = J[c2][0] * J[c1][1] - J[c2][1] * J[c1][0];
        detJ += v * v;
      }
      detJ = sqrt(detJ);
      double nrm[3] = {0.0, 0.0, 0.0};
      if (F.adv) {
        const int el = F.face_ele[f] - F.base;
        if (el < 0 || el >= F.E) {
          set_err(F.err, FL_ERR_ARG, f);
          continue;
        }
        double cf[3] = {0.0, 0.0, 0.0}, ce[3] = {0.0, 0.0, 0.0}, ow[3];
        for (int j = 0; j < 3; ++j)
          for (int a = 0; a < 3; ++a) cf[a] += Xf[j][a];
        for (int j = 0; j < 4; ++j) {
          const int v = F.xnd[4 * (int64_t)el + j];
          for (int a = 0; a < 3; ++a) ce[a] += F.X[3 * (int64_t)v + a];
        }
        for (int a = 0; a < 3; ++a) ow[a] = cf[a] / 3.0 - ce[a] / 4.0;
        double n[3] = {J[1][0] * J[2][1] - J[2][0] * J[1][1], J[2][0] * J[0][1] - J[0][0] * J[2][1],
                       J[0][0] * J[1][1] - J[1][0] * J[0][1]};
        const double o = n[0] * ow[0] + n[1] * ow[1] + n[2] * ow[2];
        for (int a = 0; a < 3; ++a) n[a] *= o;
        const double len = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int a = 0; a < 3; ++a) nrm[a] = n[a] / len;
      }
      double Tf[6];
      for (int j = 0; j < floc; ++j) Tf[j] = F.t ? F.t[fn[j]] : 0.0;
      double Madd[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, Radd = 0.0;
      if (F.adv) {
        // add_advection_face_cg: A_ij = sum_g (N_i N_j) detwei_g (u_g . n)
        double A[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int g = 0; g < F.ngi; ++g) {
          double N[6], Nu[3];
          face_shape(floc, F.ql[g], N);
          face_shape(3, F.ql[g], Nu);
          double un = 0.0;
          for (int a = 0; a < 3; ++a) {
            double uq = 0.0;
            for (int k = 0; k < 3; ++k) uq += F.u[3 * (int64_t)xv[k] + a] * Nu[k];
            un += uq * nrm[a];
          }
          const double w = (detJ * F.qw[g]) * un;
          for (int j = 0; j < floc; ++j) A[j] += (N[li] * N[j]) * w;
        }
        if (F.use_dt) {
          if (ty == 2) {
            const double* gv = F.bc1 + (int64_t)floc * f;
            double sdiff = 0.0;
            for (int j = 0; j < floc; ++j) sdiff += A[j] * (gv[j] - Tf[j]);
            Radd = Radd - F.theta * sdiff;
          } else {
            for (int j = 0; j < floc; ++j) Madd[j] = Madd[j] + F.dt_theta * A[j];
          }
        }
        double st = 0.0;
        for (int j = 0; j < floc; ++j) st += A[j] * Tf[j];
        Radd = Radd - st;
      }
      if (dface) {
        // add_diffusivity_face_cg: rhs += shape_rhs(N, detwei g_q); robin also
        // int N_i N_j g2 into the matrix (dt theta) and its product with t out of the rhs
        const double* g1 = F.bc1 + (int64_t)floc * f;
        const double* g2 = ty == 4 ? F.bc2 + (int64_t)floc * f : nullptr;
        double sr = 0.0, Rm[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (int g = 0; g < F.ngi; ++g) {
          double N[6];
          face_shape(floc, F.ql[g], N);
          const double dw = detJ * F.qw[g];
          double gq = 0.0;
          for (int k = 0; k < floc; ++k) gq += g1[k] * N[k];
          sr += N[li] * (dw * gq);
          if (g2) {
            double hq = 0.0;
            for (int k = 0; k < floc; ++k) hq += g2[k] * N[k];
            const double w = dw * hq;
            for (int j = 0; j < floc; ++j) Rm[j] += (N[li] * N[j]) * w;
          }
        }
        Radd = Radd + sr;
        if (g2) {
          if (F.use_dt)
            for (int j = 0; j < floc; ++j) Madd[j] = Madd[j] + F.dt_theta * Rm[j];
          double st = 0.0;
          for (int j = 0; j < floc; ++j) st += Rm[j] * Tf[j];
          Radd = Radd - st;
        }
      }
      // addto(matrix, face_nodes, face_nodes, matrix_addto); addto(rhs, ...)
      const int rb = F.findrm[i], re = F.findrm[i + 1];
      for (int j = 0; j < floc; ++j) {
        if (Madd[j] == 0.0) continue;
        const int p = csr_find(F.colm, rb, re, fn[j]);
        if (p < 0) {
          set_err(F.err, FL_ERR_OUTSIDE_PATTERN, i);
          continue;
        }
        F.val[p] += Madd[j];
      }
      F.rhs[i] += Radd;
    }
  }
}

static int advdif_faces(fl_mesh_t* m, const fl_advdif_params* p, const fl_face_bcs* fb, const fl_fields* f,
                        double* val, double* rhs, cudaStream_t s) {
  FL_CHECK_ARG(m && p && fb && f && val && rhs, "null argument");
  FL_CHECK_ARG(fb->nfaces >= 0, "nfaces");
  FL_CHECK_ARG(fb->index_base == 0 || fb->index_base == 1, "index_base");
  FL_CHECK_ARG(fb->floc == (m->loc == 4 ? 3 : 6), "floc must be 3 for a P1 field mesh, 6 for P2");
  const bool adv = p->have_advection && p->integrate_advection_by_parts;
  const bool diff = p->have_diffusivity != 0;
  if (fb->nfaces == 0 || !(adv || diff)) return FL_OK;  // (:608-611)
  FL_CHECK_ARG(fb->faces && fb->xfaces, "faces and xfaces");
  FL_CHECK_ARG(!adv || (fb->face_ele && f->velocity), "advection by parts needs face_ele and the velocity");
  FaceAsmArgs F{};
  F.ngi = tri_rule(p->quad_degree, F.ql, F.qw);
  FL_CHECK_ARG(F.ngi > 0, "quadrature degree 1..4");
  FL_TRY(node_face_lists(m, fb->nfaces, fb->floc, fb->faces, fb->index_base, s));
  F.N = m->N;
  F.floc = fb->floc;
  F.base = fb->index_base;
  F.E = m->E;
  F.fptr = m->face_ptr.p;
  F.flist = m->face_list.p;
  F.faces = fb->faces;
  F.xfaces = fb->xfaces;
  F.face_ele = fb->face_ele;
  F.bc_type = fb->bc_type;
  F.bc1 = fb->bc_value;
  F.bc2 = fb->bc_value2;
  F.xnd = m->xndglno.p;
  F.X = m->coords.p;
  F.u = f->velocity;
  F.t = f->t;
  F.findrm = m->findrm.p;
  F.colm = m->colm.p;
  F.val = val;
  F.rhs = rhs;
  F.theta = p->theta;
  F.dt_theta = p->dt * p->theta;
  F.use_dt = fabs(F.dt_theta) > 2.220446049250313e-16;
  F.adv = adv;
  F.diff = diff;
  F.err = m->err.p;
  k_advdif_faces<<<grid_for(m->N, 128), 128, 0, s>>>(F);
  FL_TRY_CUDA(cudaGetLastError());
  return check_err(m->err.p, s,
                   "surface loop: a face is invalid, has a weak Dirichlet condition with a diffusivity "
                   "(FLExit in the reference), lacks its boundary values, or adds outside the sparsity pattern");
}

}  // namespace fl

extern "C" int fl_dev_assemble_advdif_faces(fl_mesh m, const fl_advdif_params* p, const fl_face_bcs* fb,
                                            const fl_fields* f, double* val, double* rhs, void* stream) {
  FL_CHECK_ARG(m, "null mesh");
  return fl::advdif_faces(m, p, fb, f, val, rhs, pick_stream(m, stream));
}

extern "C" int fl_gpu_assemble_advdif_faces(fl_mesh m, const fl_advdif_params* p, const fl_face_bcs* fb,
                                            const fl_fields* f, double* val, double* rhs) {
  using namespace fl;
  FL_CHECK_ARG(m && p && fb && f && val && rhs, "null argument");
  FL_CHECK_ARG(fb->nfaces >= 0 && fb->floc > 0 && fb->floc <= 6, "nfaces and floc");
  cudaStream_t s = m->stream;
  const int nf = fb->nfaces, floc = fb->floc;
  // device copies of the face arrays and fields in the mesh's grow-only
  // staging buffers (calls on one handle share them)
  const size_t ni = (size_t)nf * (floc + 3 + 2), nd = (size_t)nf * floc * 2;
  FL_TRY(m->st_nodes.reserve(ni));
  FL_TRY(m->st_g.reserve(nd));
  int32_t* d_faces = m->st_nodes.p;
  int32_t* d_xfaces = d_faces + (size_t)nf * floc;
  int32_t* d_fe = d_xfaces + (size_t)nf * 3;
  int32_t* d_bt = d_fe + nf;
  double* d_b1 = m->st_g.p;
  double* d_b2 = m->st_g.p + (size_t)nf * floc;
  if (nf > 0) {
    FL_CHECK_ARG(fb->faces && fb->xfaces, "faces and xfaces");
    FL_TRY_CUDA(cudaMemcpyAsync(d_faces, fb->faces, sizeof(int32_t) * nf * floc, cudaMemcpyHostToDevice, s));
    FL_TRY_CUDA(cudaMemcpyAsync(d_xfaces, fb->xfaces, sizeof(int32_t) * nf * 3, cudaMemcpyHostToDevice, s));
    if (fb->face_ele)
      FL_TRY_CUDA(cudaMemcpyAsync(d_fe, fb->face_ele, sizeof(int32_t) * nf, cudaMemcpyHostToDevice, s));
    if (fb->bc_type)
      FL_TRY_CUDA(cudaMemcpyAsync(d_bt, fb->bc_type, sizeof(int32_t) * nf, cudaMemcpyHostToDevice, s));
    if (fb->bc_value)
      FL_TRY_CUDA(cudaMemcpyAsync(d_b1, fb->bc_value, sizeof(double) * nf * floc, cudaMemcpyHostToDevice, s));
    if (fb->bc_value2)
      FL_TRY_CUDA(cudaMemcpyAsync(d_b2, fb->bc_value2, sizeof(double) * nf * floc, cudaMemcpyHostToDevice, s));
  }
  fl_face_bcs dfb = *fb;
  dfb.faces = d_faces;
  dfb.xfaces = d_xfaces;
  dfb.face_ele = fb->face_ele ? d_fe : nullptr;
  dfb.bc_type = fb->bc_type ? d_bt : nullptr;
  dfb.bc_value = fb->bc_value ? d_b1 : nullptr;
  dfb.bc_value2 = fb->bc_value2 ? d_b2 : nullptr;
  FL_TRY(m->st_val.reserve(m->nnz));
  FL_TRY(m->st_rhs.reserve(m->N));
  FL_TRY_CUDA(cudaMemcpyAsync(m->st_val.p, val, sizeof(double) * m->nnz, cudaMemcpyHostToDevice, s));
  FL_TRY_CUDA(cudaMemcpyAsync(m->st_rhs.p, rhs, sizeof(double) * m->N, cudaMemcpyHostToDevice, s));
  fl_fields df{};
  if (f->t) {
    FL_TRY(m->st_t.reserve(m->N));
    FL_TRY_CUDA(cudaMemcpyAsync(m->st_t.p, f->t, sizeof(double) * m->N, cudaMemcpyHostToDevice, s));
    df.t = m->st_t.p;
  }
  if (f->velocity) {
    FL_TRY(m->st_u.reserve((size_t)3 * m->Nx));
    FL_TRY_CUDA(cudaMemcpyAsync(m->st_u.p, f->velocity, sizeof(double) * 3 * m->Nx, cudaMemcpyHostToDevice, s));
    df.velocity = m->st_u.p;
  }
  FL_TRY(advdif_faces(m, p, &dfb, &df, m->st_val.p, m->st_rhs.p, s));
  FL_TRY_CUDA(cudaMemcpyAsync(val, m->st_val.p, sizeof(double) * m->nnz, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaMemcpyAsync(rhs, m->st_rhs.p, sizeof(double) * m->N, cudaMemcpyDeviceToHost, s));
  FL_TRY_CUDA(cudaStreamSynchronize(s));
  return FL_OK;
}
