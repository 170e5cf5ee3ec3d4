// fl_oracle.cpp -- CPU restatement of Fluidity's CG assembly + Krylov hot path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the checker for the GPU library and
// the timed CPU baseline ("port" of the reference algorithm).  Nothing in the
// product (fluidity_gb300/) links, loads or calls it.  Only tests/, the smoke
// check and bench.py's CPU-baseline leg may use it.
//
// Parity status: the reference (Fortran 90 + PETSc) cannot be compiled in this
// environment (no Fortran compiler, no PETSc).  The restatement is pinned
// against the reference's own known-answer unit tests (quadrature exactness,
// femtools/tests/test_quadrature.F90; shape-function exactness,
// femtools/tests/test_shape_functions.F90; the Jacobian known answer,
// femtools/tests/test_jacobian.F90; colouring validity and partition,
// femtools/tests/test_colouring.F90) and against analytic facts (scipy direct
// solves, MMS convergence order).  Assembled entries and Krylov iteration
// counts are not pinned by any reference test.
//
// Every routine cites the reference file:line it restates.  Indices are
// 0-based inside this file; the Python wrapper converts at the boundary.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Reference element: tetrahedral quadrature.
// femtools/Quadrature.F90:649-735 (construct_tet_quadratures) expanded by
// expand_quadrature_template (Quadrature.F90:572-605) with the permutation
// tables of construct_tet_permutations (Quadrature.F90:1635-1736).
// Point k of a generator with permutation column p(:,k) has barycentric
// coordinate l(j) = coords(p(j,k)).  Literals are real(8) because the
// reference is built with -fdefault-real-8.
// ---------------------------------------------------------------------------
struct Quad {
  int degree = 0, ngi = 0;
  double l[16][4];
  double w[16];
};

void add_points(Quad& q, const int (*perm)[4], int np, double weight,
                const double* coords) {
  for (int k = 0; k < np; ++k) {
    for (int j = 0; j < 4; ++j) q.l[q.ngi][j] = coords[perm[k][j] - 1];
    q.w[q.ngi] = weight;
    ++q.ngi;
  }
}

// Permutation 7 (1 point), 8 (4 points), 9 (6 points); columns as in
// Quadrature.F90:1722-1736.
const int kPerm7[1][4] = {{1, 1, 1, 1}};
const int kPerm8[4][4] = {{1, 1, 1, 2}, {1, 1, 2, 1}, {1, 2, 1, 1}, {2, 1, 1, 1}};
const int kPerm9[6][4] = {{1, 1, 2, 2}, {1, 2, 1, 2}, {1, 2, 2, 1},
                          {2, 1, 1, 2}, {2, 1, 2, 1}, {2, 2, 1, 1}};

// make_quadrature picks the template of minimum degree >= requested
// (Quadrature.F90:318).  Degrees 1..4 are the rules on the CG hot path.
bool make_tet_quad(int degree, Quad& q) {
  q = Quad();
  if (degree <= 1) {  // Str71, 1 point
    double c[1] = {0.25};
    add_points(q, kPerm7, 1, 0.166666666666666666666666666666666, c);
    q.degree = 1;
  } else if (degree == 2) {  // Str71, 4 points
    double c[2];
    c[0] = 0.138196601125010515179541316563436;
    c[1] = 1.0 - 3.0 * c[0];
    add_points(q, kPerm8, 4, 0.041666666666666666666666666666666, c);
    q.degree = 2;
  } else if (degree == 3) {  // Str71, 5 points
    double c1[1] = {0.25};
    add_points(q, kPerm7, 1, -0.133333333333333333333333333333333, c1);
    double c[2];
    c[0] = 0.166666666666666666666666666666666;
    c[1] = 1.0 - 3.0 * c[0];
    add_points(q, kPerm8, 4, 0.075, c);
    q.degree = 3;
  } else if (degree == 4) {  // kea86, 11 points (one negative weight)
    double c1[1] = {0.25};
    add_points(q, kPerm7, 1, -0.013155555555555555555555555555555, c1);
    double c[2];
    c[0] = 0.0714285714285714285714285714285714;
    c[1] = 1.0 - 3.0 * c[0];
    add_points(q, kPerm8, 4, 7.62222222222222222222222222222222E-3, c);
    c[0] = 0.399403576166799204996102147461640;
    c[1] = 0.5 - c[0];
    add_points(q, kPerm9, 6, 0.0248888888888888888888888888888888, c);
    q.degree = 4;
  } else {
    return false;
  }
  return true;
}

// ---------------------------------------------------------------------------
// Lagrange simplex shape functions.
// Local node order: femtools/Element_Numbering.F90:389-472
// (number_tets_lagrange); node i has barycentric "counts" l(1..4).
// Polynomials: Shape_Functions.F90:331 (lagrange_polynomial) -- the 1-D factor
// for count c and degree d is prod_{k<c} (x - k/d) / (c/d - k/d).
// Derivatives w.r.t. L1..L3 with L4 dependent: Elements.F90:615-690
// (eval_dshape_simplex) and diffl4 = -1 (Elements.F90:693-717).
// ---------------------------------------------------------------------------
struct Shape {
  int degree = 0, loc = 0, ngi = 0;
  int counts[10][4];
  double n[10][16];
  double dn[10][16][3];
};

void tet_counts(int degree, int (*counts)[4], int* loc) {
  int l[4] = {degree, 0, 0, 0};
  int cnt = 0;
  while (true) {
    for (int j = 0; j < 4; ++j) counts[cnt][j] = l[j];
    ++cnt;
    if (l[3] == degree) break;
    l[1] += 1;
    for (int j = 1; j <= 2; ++j) {
      int tail = 0;
      for (int k = j + 1; k < 4; ++k) tail += l[k];
      if (l[j] > degree - tail) {
        l[j] = 0;
        l[j + 1] += 1;
      }
    }
    l[0] = degree - (l[1] + l[2] + l[3]);
  }
  *loc = cnt;
}

double lag1d(int c, int degree, double x) {
  double dx = 1.0 / degree, v = 1.0, norm = 1.0;
  for (int k = 0; k < c; ++k) {
    v *= (x - k * dx);
    norm *= (c * dx - k * dx);
  }
  return v / norm;
}

double dlag1d(int c, int degree, double x) {
  double dx = 1.0 / degree, norm = 1.0, s = 0.0;
  for (int k = 0; k < c; ++k) norm *= (c * dx - k * dx);
  for (int m = 0; m < c; ++m) {
    double p = 1.0;
    for (int k = 0; k < c; ++k)
      if (k != m) p *= (x - k * dx);
    s += p;
  }
  return s / norm;
}

void make_shape(int degree, const Quad& q, Shape& s) {
  s = Shape();
  s.degree = degree;
  s.ngi = q.ngi;
  tet_counts(degree, s.counts, &s.loc);
  for (int i = 0; i < s.loc; ++i) {
    const int* c = s.counts[i];
    for (int g = 0; g < q.ngi; ++g) {
      const double* l = q.l[g];
      double p[4], dp[4];
      for (int j = 0; j < 4; ++j) {
        p[j] = lag1d(c[j], degree, l[j]);
        dp[j] = dlag1d(c[j], degree, l[j]);
      }
      s.n[i][g] = p[0] * p[1] * p[2] * p[3];
      for (int d = 0; d < 3; ++d) {
        double v = dp[d] * p[3] + (-1.0) * dp[3] * p[d];
        for (int j = 0; j < 3; ++j)
          if (j != d) v *= p[j];
        s.dn[i][g][d] = v;
      }
    }
  }
}

// Local position of the vertices and edges of a P2 tet in the
// number_tets_lagrange order: vertex v has count 2 at v; edge (a,b) has
// counts 1 at a and b.
int local_of_counts(const Shape& s, const int* c) {
  for (int i = 0; i < s.loc; ++i) {
    bool eq = true;
    for (int j = 0; j < 4; ++j) eq = eq && (s.counts[i][j] == c[j]);
    if (eq) return i;
  }
  return -1;
}

// ---------------------------------------------------------------------------
// Geometry cache for linear simplex coordinates.
// femtools/Transform_elements.F90:227-306 (construct_cache):
//   J_T = X_val . dn(:,1,:)            (dim x dim)
//   invJ(i,k) = cofactor via cyc3      (Transform_elements.F90:285-293)
//   detJ = dot(J_T(:,1), invJ(:,1)); invJ = invJ / detJ
// and the use of the cache in transform_to_physical_full
// (Transform_elements.F90:788-829): dshape(:,gi,:) = dn(:,gi,:) . invJ^T,
// detwei = |detJ| * w.
// ---------------------------------------------------------------------------
const int cyc3[5] = {0, 1, 2, 0, 1};

struct Geo {
  double JT[3][3], invJ[3][3], detJ;
};

void element_geometry(const double* X /*3 x 4, column = vertex*/,
                      const Shape& xs, Geo& g) {
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double s = 0.0;
      for (int i = 0; i < 4; ++i) s += X[3 * i + a] * xs.dn[i][0][b];
      g.JT[a][b] = s;
    }
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k)
      g.invJ[i][k] = g.JT[cyc3[i + 1]][cyc3[k + 1]] * g.JT[cyc3[i + 2]][cyc3[k + 2]] -
                     g.JT[cyc3[i + 2]][cyc3[k + 1]] * g.JT[cyc3[i + 1]][cyc3[k + 2]];
  g.detJ = g.JT[0][0] * g.invJ[0][0] + g.JT[1][0] * g.invJ[1][0] + g.JT[2][0] * g.invJ[2][0];
  for (int i = 0; i < 3; ++i)
    for (int k = 0; k < 3; ++k) g.invJ[i][k] = g.invJ[i][k] / g.detJ;
}

// ---------------------------------------------------------------------------
// CSR helpers.  csr_sparsity_pos (femtools/Sparse_Tools.F90:2411-2517) is a
// bisection over the sorted row; csr_addto (Sparse_Tools.F90:2631-2655) skips
// exact zeros and aborts when the entry is outside the pattern.
// ---------------------------------------------------------------------------
inline int64_t csr_pos(const int64_t* findrm, const int* colm, int i, int j) {
  int64_t lo = findrm[i], hi = findrm[i + 1] - 1;
  while (lo <= hi) {
    int64_t mid = (lo + hi) / 2;
    int c = colm[mid];
    if (c == j) return mid;
    if (c < j) lo = mid + 1;
    else hi = mid - 1;
  }
  return -1;
}

}  // namespace

extern "C" {

// Status codes shared with the Python wrapper.
enum { ORC_OK = 0, ORC_ERR_ARG = 1, ORC_ERR_OUTSIDE_PATTERN = 3 };

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// Quadrature table for a requested degree (Quadrature.F90:164-500).
int orc_tet_quadrature(int degree, int* ngi, int* actual_degree, double* l, double* w) {
  Quad q;
  if (!make_tet_quad(degree, q)) return ORC_ERR_ARG;
  *ngi = q.ngi;
  *actual_degree = q.degree;
  for (int g = 0; g < q.ngi; ++g) {
    for (int j = 0; j < 4; ++j) l[4 * g + j] = q.l[g][j];
    w[g] = q.w[g];
  }
  return ORC_OK;
}

// Shape functions n(loc,ngi) and dn(loc,ngi,3), row-major [i][g][d].
int orc_tet_shape(int degree, int quad_degree, int* loc, int* ngi, double* n, double* dn) {
  Quad q;
  if (!make_tet_quad(quad_degree, q) || degree < 1 || degree > 2) return ORC_ERR_ARG;
  Shape s;
  make_shape(degree, q, s);
  *loc = s.loc;
  *ngi = s.ngi;
  for (int i = 0; i < s.loc; ++i)
    for (int g = 0; g < s.ngi; ++g) {
      n[i * s.ngi + g] = s.n[i][g];
      for (int d = 0; d < 3; ++d) dn[(i * s.ngi + g) * 3 + d] = s.dn[i][g][d];
    }
  return ORC_OK;
}

// Reference-node counts in local order (Element_Numbering.F90:389-472).
int orc_tet_counts(int degree, int* counts /*loc*4*/) {
  int c[10][4], loc = 0;
  if (degree < 1 || degree > 2) return -1;
  tet_counts(degree, c, &loc);
  for (int i = 0; i < loc; ++i)
    for (int j = 0; j < 4; ++j) counts[4 * i + j] = c[i][j];
  return loc;
}

// Jacobian known answer of femtools/tests/test_jacobian.F90: a P1 triangle
// embedded in 3-D.  compute_jacobian for dim < xdim forms J (dim x xdim) and
// detwei = sqrt(det(J J^T)) * w; restated here for the triangle only so the
// test's known answer sum(detwei) = sqrt(2) can pin the transform arithmetic.
double orc_triangle_detwei_sum(const double* X /*3 x 3, column=vertex*/) {
  // Degree-4 triangle rule weights sum to 1/2 (reference triangle area); for an
  // affine triangle detwei is constant * w, so only the weight sum matters.
  double e1[3], e2[3];
  for (int a = 0; a < 3; ++a) {
    e1[a] = X[3 * 0 + a] - X[3 * 2 + a];
    e2[a] = X[3 * 1 + a] - X[3 * 2 + a];
  }
  double g11 = e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2];
  double g22 = e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2];
  double g12 = e1[0] * e2[0] + e1[1] * e2[1] + e1[2] * e2[2];
  return std::sqrt(g11 * g22 - g12 * g12) * 0.5;
}

// Element geometry cache for all elements (Transform_elements.F90:227-306).
// out: JT[9*E], invJ[9*E] (row-major [a][b]), detJ[E].
int orc_transform_cache(int E, const int* ndglno_x /*4*E*/, const double* coords,
                        double* JT, double* invJ, double* detJ) {
  Quad q;
  make_tet_quad(1, q);
  Shape xs;
  make_shape(1, q, xs);
#pragma omp parallel for schedule(static)
  for (int e = 0; e < E; ++e) {
    double X[12];
    for (int i = 0; i < 4; ++i)
      for (int a = 0; a < 3; ++a) X[3 * i + a] = coords[3 * (int64_t)ndglno_x[4 * (int64_t)e + i] + a];
    Geo g;
    element_geometry(X, xs, g);
    for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b) {
        JT[9 * (int64_t)e + 3 * a + b] = g.JT[a][b];
        invJ[9 * (int64_t)e + 3 * a + b] = g.invJ[a][b];
      }
    detJ[e] = g.detJ;
  }
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// make_sparsity (Sparsity_Patterns.F90:47-85 -> make_sparsity_lists :299-379 ->
// lists2csr_sparsity :381-430): every (row node, column node) pair sharing an
// element, rows ascending (insert_ascending), centrm = diagonal position.
// Two-call protocol: with colm == nullptr only the entry count is returned.
// ---------------------------------------------------------------------------
int64_t orc_make_sparsity(int nrows, int E, int loc, const int* ndglno,
                          int64_t* findrm, int* colm, int64_t cap, int64_t* centrm) {
  std::vector<std::vector<int>> rows(nrows);
  for (int e = 0; e < E; ++e) {
    const int* en = ndglno + (int64_t)loc * e;
    for (int i = 0; i < loc; ++i) {
      std::vector<int>& r = rows[en[i]];
      for (int j = 0; j < loc; ++j) {
        auto it = std::lower_bound(r.begin(), r.end(), en[j]);
        if (it == r.end() || *it != en[j]) r.insert(it, en[j]);
      }
    }
  }
  int64_t nnz = 0;
  for (int i = 0; i < nrows; ++i) nnz += (int64_t)rows[i].size();
  if (!colm || cap < nnz) return nnz;
  int64_t p = 0;
  for (int i = 0; i < nrows; ++i) {
    findrm[i] = p;
    centrm[i] = -1;
    for (int c : rows[i]) {
      if (c == i) centrm[i] = p;
      colm[p++] = c;
    }
  }
  findrm[nrows] = p;
  return nnz;
}

// ---------------------------------------------------------------------------
// COLOURING_CG1 (Colouring.F90:85-154 in an OpenMP build): the element graph
// is the second-order sparsity C^T C of the P0 mesh over the topology mesh
// (elements sharing a vertex; Sparsity_Patterns.F90:87-148), coloured greedily
// in element order considering lower-numbered neighbours only
// (colour_sparsity, Colouring.F90:159-199).  Colours are 1-based; colour sets
// iterate in ascending element id (colour_sets :250-262, Judy1 ascending).
// ---------------------------------------------------------------------------
int orc_colour_cg1(int E, int nv_loc, const int* ndglno_vertices, int nvert, int* colour) {
  std::vector<int64_t> ptr(nvert + 1, 0);
  for (int64_t k = 0; k < (int64_t)E * nv_loc; ++k) ptr[ndglno_vertices[k] + 1]++;
  for (int v = 0; v < nvert; ++v) ptr[v + 1] += ptr[v];
  std::vector<int> elems(ptr[nvert]);
  std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
  for (int e = 0; e < E; ++e)
    for (int i = 0; i < nv_loc; ++i) elems[fill[ndglno_vertices[(int64_t)nv_loc * e + i]]++] = e;
  int ncol = 0;
  std::vector<int> mark(64, -1);
  for (int e = 0; e < E; ++e) {
    for (int i = 0; i < nv_loc; ++i) {
      int v = ndglno_vertices[(int64_t)nv_loc * e + i];
      for (int64_t k = ptr[v]; k < ptr[v + 1]; ++k) {
        int f = elems[k];
        if (f < e) {
          int c = colour[f];
          if (c >= (int)mark.size()) mark.resize(2 * c + 2, -1);
          mark[c] = e;
        }
      }
    }
    int c = 1;
    while (c < (int)mark.size() && mark[c] == e) ++c;
    if (c >= (int)mark.size()) mark.resize(2 * c + 2, -1);
    colour[e] = c;
    ncol = std::max(ncol, c);
  }
  return ncol;
}

// ---------------------------------------------------------------------------
// make_global_numbering for a P2 tet mesh from a P1 connectivity, serial case
// (Global_Numbering.F90:291-634): vertices are renumbered in first-touch
// element order (:460-493), then each edge (node, node2>node) is numbered in
// order of old node ascending and NNList row ascending (:497-634; NNList from
// POSINM, Sparse_Tools.F90:462-591, rows sorted ascending).  Output ndglno2 is
// 0-based in number_tets_lagrange local order; returns the node count.
// ---------------------------------------------------------------------------
int orc_make_global_numbering_p2(int nvert, int E, const int* ndglno1, int* ndglno2) {
  Quad q;
  make_tet_quad(1, q);
  Shape s2;
  make_shape(2, q, s2);
  int vpos[4], epos[4][4];
  for (int a = 0; a < 4; ++a) {
    int c[4] = {0, 0, 0, 0};
    c[a] = 2;
    vpos[a] = local_of_counts(s2, c);
    for (int b = 0; b < 4; ++b) {
      if (a == b) { epos[a][b] = -1; continue; }
      int cc[4] = {0, 0, 0, 0};
      cc[a] = 1;
      cc[b] = 1;
      epos[a][b] = local_of_counts(s2, cc);
    }
  }
  std::fill(ndglno2, ndglno2 + (int64_t)10 * E, -1);
  std::vector<int> node_map(nvert, -1);
  int n = 0;
  for (int e = 0; e < E; ++e)
    for (int j = 0; j < 4; ++j) {
      int v = ndglno1[4 * (int64_t)e + j];
      if (node_map[v] < 0) node_map[v] = n++;
      ndglno2[10 * (int64_t)e + vpos[j]] = node_map[v];
    }
  // NEList: elements of each node, ascending.
  std::vector<int64_t> ptr(nvert + 1, 0);
  for (int64_t k = 0; k < 4 * (int64_t)E; ++k) ptr[ndglno1[k] + 1]++;
  for (int v = 0; v < nvert; ++v) ptr[v + 1] += ptr[v];
  std::vector<int> elems(ptr[nvert]);
  std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
  for (int e = 0; e < E; ++e)
    for (int i = 0; i < 4; ++i) elems[fill[ndglno1[4 * (int64_t)e + i]]++] = e;
  // NNList rows: sorted unique neighbours.
  std::vector<int> nbr;
  for (int node = 0; node < nvert; ++node) {
    nbr.clear();
    for (int64_t k = ptr[node]; k < ptr[node + 1]; ++k) {
      int e = elems[k];
      for (int i = 0; i < 4; ++i) nbr.push_back(ndglno1[4 * (int64_t)e + i]);
    }
    std::sort(nbr.begin(), nbr.end());
    nbr.erase(std::unique(nbr.begin(), nbr.end()), nbr.end());
    for (int node2 : nbr) {
      if (node2 <= node) continue;
      // Every element of node2 that also contains node gets the edge number.
      for (int64_t k = ptr[node2]; k < ptr[node2 + 1]; ++k) {
        int e = elems[k];
        const int* en = ndglno1 + 4 * (int64_t)e;
        int a = -1, b = -1;
        for (int i = 0; i < 4; ++i) {
          if (en[i] == node) a = i;
          if (en[i] == node2) b = i;
        }
        if (a >= 0 && b >= 0) ndglno2[10 * (int64_t)e + epos[a][b]] = n;
      }
      n += 1;
    }
  }
  return n;
}

// ---------------------------------------------------------------------------
// Element assembly of the CG advection-diffusion equation in acceleration
// form (assemble/Advection_Diffusion_CG.F90:702-865 and term routines
// :867-941 mass, :943-1127 advection (not integrated by parts, no
// stabilisation, default equation type), :1143-1162 absorption, :1164-1202
// diffusivity, :1129-1141 source) followed by addto (Sparse_Tools.F90:2680).
// The element loop visits colour sets in order, elements ascending within a
// colour (Advection_Diffusion_CG.F90:582-598); with no colouring given it is
// the serial build's single colour holding all elements.
// ---------------------------------------------------------------------------
struct OrcAdvDifParams {
  double theta, dt, beta;
  int have_mass, lump_mass, have_advection, have_diffusivity, isotropic;
  int have_source, have_absorption, quad_degree, t_degree, u_degree;
  double diffusivity[9];  // constant tensor, row-major
  int by_parts;           // integrate_advection_by_parts
  int pad;
};

int orc_assemble_advdif(const OrcAdvDifParams* P, int E, const int* ndglno_t, int nt,
                        const int* ndglno_x, const double* coords,
                        const int* ndglno_u, const double* velocity,
                        const double* T, const double* source, const double* absorption,
                        const int64_t* findrm, const int* colm, double* val, double* rhs,
                        int ncolours, const int64_t* colour_ptr, const int* colour_elems,
                        int nthreads) {
  Quad q;
  if (!make_tet_quad(P->quad_degree, q)) return ORC_ERR_ARG;
  Shape ts, xs, us;
  make_shape(P->t_degree, q, ts);
  make_shape(1, q, xs);
  make_shape(P->have_advection ? P->u_degree : 1, q, us);
  const int loc = ts.loc, ngi = q.ngi, uloc = us.loc;
  const double dt_theta = P->dt * P->theta;
  // epsilon(0.0): the literal is real(8) under -fdefault-real-8.
  const double eps0 = 2.220446049250313e-16;
  int status = ORC_OK;
  // zero(matrix); zero(rhs)  (Advection_Diffusion_CG.F90:560-561)
  std::memset(val, 0, sizeof(double) * (size_t)(findrm[nt] - findrm[0]));
  std::memset(rhs, 0, sizeof(double) * (size_t)nt);

  std::vector<int64_t> dflt_ptr;
  std::vector<int> dflt_elems;
  // Without a colouring the loop is the serial build's single colour holding
  // every element (Colouring.F90:145-151), and it must run on one thread.
  const bool serial = ncolours <= 0;
  if (ncolours <= 0) {
    ncolours = 1;
    dflt_ptr = {0, E};
    dflt_elems.resize(E);
    for (int e = 0; e < E; ++e) dflt_elems[e] = e;
    colour_ptr = dflt_ptr.data();
    colour_elems = dflt_elems.data();
  }
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif

#pragma omp parallel if (!serial)
  {
    for (int clr = 0; clr < ncolours; ++clr) {
#pragma omp for schedule(static)
      for (int64_t idx = colour_ptr[clr]; idx < colour_ptr[clr + 1]; ++idx) {
        const int e = colour_elems[idx];
        // Step 1: transform (cached linear-simplex geometry).
        double X[12];
        for (int i = 0; i < 4; ++i)
          for (int a = 0; a < 3; ++a) X[3 * i + a] = coords[3 * (int64_t)ndglno_x[4 * (int64_t)e + i] + a];
        Geo g;
        element_geometry(X, xs, g);
        double detwei[16];
        for (int gi = 0; gi < ngi; ++gi) detwei[gi] = std::fabs(g.detJ) * q.w[gi];
        double dt_t[10][16][3];
        for (int gi = 0; gi < ngi; ++gi)
          for (int i = 0; i < loc; ++i)
            for (int a = 0; a < 3; ++a) {
              double s = 0.0;
              for (int b = 0; b < 3; ++b) s += ts.dn[i][gi][b] * g.invJ[a][b];
              dt_t[i][gi][a] = s;
            }
        const int* tn = ndglno_t + (int64_t)loc * e;
        double Te[10];
        for (int i = 0; i < loc; ++i) Te[i] = T ? T[tn[i]] : 0.0;
        double M[10][10] = {}, R[10] = {};

        // Mass (Advection_Diffusion_CG.F90:867-941): shape_shape (FETools.F90:206).
        if (P->have_mass) {
          for (int i = 0; i < loc; ++i)
            for (int j = 0; j < loc; ++j) {
              double s = 0.0;
              for (int gi = 0; gi < ngi; ++gi) s += ts.n[i][gi] * ts.n[j][gi] * detwei[gi];
              if (P->lump_mass) M[i][i] += s;
              else M[i][j] += s;
            }
        }
        // Advection (Advection_Diffusion_CG.F90:1019-1113).  Not by parts:
        // A = shape_vector_dot_dshape(N, u_q, dN, detwei)   (FETools.F90:749)
        //   + beta * shape_shape(N, N, div(u)_q * detwei); by parts see below.
        // matrix += dt_theta*A; rhs -= A.T_e (:1117-1125).
        if (P->have_advection) {
          const int* un = ndglno_u + (int64_t)uloc * e;
          double uq[16][3] = {}, divu[16] = {};
          for (int gi = 0; gi < ngi; ++gi)
            for (int a = 0; a < 3; ++a) {
              double s = 0.0;
              for (int i = 0; i < uloc; ++i) s += velocity[3 * (int64_t)un[i] + a] * us.n[i][gi];
              uq[gi][a] = s;
            }
          // the divergence term: beta (not by parts) or 1 - beta (by parts)
          const double bcoef = P->by_parts ? 1.0 - P->beta : P->beta;
          if (std::fabs(bcoef) > eps0) {
            // ele_div_at_quad with du_t = dN_u . invJ^T
            for (int gi = 0; gi < ngi; ++gi) {
              double s = 0.0;
              for (int i = 0; i < uloc; ++i)
                for (int a = 0; a < 3; ++a) {
                  double d = 0.0;
                  for (int b = 0; b < 3; ++b) d += us.dn[i][gi][b] * g.invJ[a][b];
                  s += velocity[3 * (int64_t)un[i] + a] * d;
                }
              divu[gi] = s;
            }
          }
          double A[10][10];
          if (P->by_parts) {
            // By parts (:1019-1057): A = -dshape_dot_vector_shape(dN, u_q, N,
            // detwei) (FETools.F90:700-721) - (1 - beta) shape_shape(N, N,
            // div(u)_q detwei)
            for (int i = 0; i < loc; ++i)
              for (int j = 0; j < loc; ++j) {
                double s = 0.0;
                for (int gi = 0; gi < ngi; ++gi) {
                  double udn = 0.0;
                  for (int a = 0; a < 3; ++a) udn += dt_t[i][gi][a] * uq[gi][a];
                  s += udn * ts.n[j][gi] * detwei[gi];
                }
                A[i][j] = -s;
              }
          } else {
            for (int i = 0; i < loc; ++i)
              for (int j = 0; j < loc; ++j) {
                double s = 0.0;
                for (int gi = 0; gi < ngi; ++gi) {
                  double udn = 0.0;
                  for (int a = 0; a < 3; ++a) udn += dt_t[j][gi][a] * uq[gi][a];
                  s += ts.n[i][gi] * udn * detwei[gi];
                }
                A[i][j] = s;
              }
          }
          if (std::fabs(bcoef) > eps0)
            for (int i = 0; i < loc; ++i)
              for (int j = 0; j < loc; ++j) {
                double s = 0.0;
                for (int gi = 0; gi < ngi; ++gi) s += ts.n[i][gi] * ts.n[j][gi] * (divu[gi] * detwei[gi]);
                if (P->by_parts) A[i][j] = A[i][j] - bcoef * s;
                else A[i][j] = A[i][j] + bcoef * s;
              }
          for (int i = 0; i < loc; ++i) {
            if (std::fabs(dt_theta) > eps0)
              for (int j = 0; j < loc; ++j) M[i][j] += dt_theta * A[i][j];
            double s = 0.0;
            for (int j = 0; j < loc; ++j) s += A[i][j] * Te[j];
            R[i] -= s;
          }
        }
        // Absorption (:1143-1162).
        if (P->have_absorption) {
          double aq[16];
          for (int gi = 0; gi < ngi; ++gi) {
            double s = 0.0;
            for (int i = 0; i < loc; ++i) s += absorption[tn[i]] * ts.n[i][gi];
            aq[gi] = s;
          }
          double A[10][10];
          for (int i = 0; i < loc; ++i)
            for (int j = 0; j < loc; ++j) {
              double s = 0.0;
              for (int gi = 0; gi < ngi; ++gi) s += ts.n[i][gi] * ts.n[j][gi] * (detwei[gi] * aq[gi]);
              A[i][j] = s;
            }
          for (int i = 0; i < loc; ++i) {
            if (std::fabs(dt_theta) > eps0)
              for (int j = 0; j < loc; ++j) M[i][j] += dt_theta * A[i][j];
            double s = 0.0;
            for (int j = 0; j < loc; ++j) s += A[i][j] * Te[j];
            R[i] -= s;
          }
        }
        // Diffusivity (:1164-1202): dshape_dot_dshape (FETools.F90:391-453)
        // for isotropic, dshape_tensor_dshape (FETools.F90:668-698) otherwise.
        if (P->have_diffusivity) {
          double K[10][10] = {};
          const double* kap = P->diffusivity;
          for (int gi = 0; gi < ngi; ++gi)
            for (int i = 0; i < loc; ++i)
              for (int j = 0; j < loc; ++j) {
                double v;
                if (P->isotropic) {
                  v = ((dt_t[i][gi][0] * dt_t[j][gi][0]) + (dt_t[i][gi][1] * dt_t[j][gi][1]) +
                       (dt_t[i][gi][2] * dt_t[j][gi][2])) * (detwei[gi] * kap[0]);
                } else {
                  double tmp[3];
                  for (int b = 0; b < 3; ++b)
                    tmp[b] = dt_t[i][gi][0] * kap[0 * 3 + b] + dt_t[i][gi][1] * kap[1 * 3 + b] +
                             dt_t[i][gi][2] * kap[2 * 3 + b];
                  v = (tmp[0] * dt_t[j][gi][0] + tmp[1] * dt_t[j][gi][1] + tmp[2] * dt_t[j][gi][2]) *
                      detwei[gi];
                }
                K[i][j] = K[i][j] + v;
              }
          for (int i = 0; i < loc; ++i) {
            if (std::fabs(dt_theta) > eps0)
              for (int j = 0; j < loc; ++j) M[i][j] += dt_theta * K[i][j];
            double s = 0.0;
            for (int j = 0; j < loc; ++j) s += K[i][j] * Te[j];
            R[i] -= s;
          }
        }
        // Source (:1129-1141): shape_rhs(N, detwei * f_q) (FETools.F90:38).
        if (P->have_source) {
          double fq[16];
          for (int gi = 0; gi < ngi; ++gi) {
            double s = 0.0;
            for (int i = 0; i < loc; ++i) s += source[tn[i]] * ts.n[i][gi];
            fq[gi] = detwei[gi] * s;
          }
          for (int i = 0; i < loc; ++i) {
            double s = 0.0;
            for (int gi = 0; gi < ngi; ++gi) s += ts.n[i][gi] * fq[gi];
            R[i] += s;
          }
        }
        // Insertion: addto(matrix, nodes, nodes, M); addto(rhs, nodes, R).
        for (int i = 0; i < loc; ++i) {
          for (int j = 0; j < loc; ++j) {
            if (M[i][j] == 0.0) continue;
            int64_t p = csr_pos(findrm, colm, tn[i], tn[j]);
            if (p < 0) {
#pragma omp atomic write
              status = ORC_ERR_OUTSIDE_PATTERN;
              continue;
            }
            val[p] += M[i][j];
          }
          rhs[tn[i]] += R[i];
        }
      }
    }
  }
  return status;
}

// ---------------------------------------------------------------------------
// The surface loop of assemble_advection_diffusion_cg (Advection_Diffusion_CG
// .F90:608-640), run after the element loop and before the strong Dirichlet
// conditions: for each surface element in order, unless its bc type is
// internal (3), assemble_advection_diffusion_face_cg (:1228-1286) with
// add_advection_face_cg (:1288-1342, advection integrated by parts only) and
// add_diffusivity_face_cg (:1344-1378), then addto of the face matrix and rhs.
// bc types (get_entire_boundary_condition order, :74-75): 0 none, 1 neumann,
// 2 weakdirichlet, 3 internal, 4 robin.  Face transform: transform_facet_to
// _physical (Transform_elements.F90:1353-1525) for a linear face: J = [X1 - X3,
// X2 - X3], detJ = |J1 x J2| summed in cyc3 order, detwei = detJ * w, normal
// = facet_normal (:1527-1553) oriented by face centroid - element centroid.
// Face quadrature: the triangle rule of the element rule's degree
// (Quadrature.F90:908-1010, construct_tri_quadratures).  Face shape functions
// in the triangle's local order (P1: vertices; P2: vertex 1, edge 12, vertex
// 2, edge 13, edge 23, vertex 3).
// ---------------------------------------------------------------------------
namespace {

struct TriRule {
  int ngi = 0;
  double l[6][3];
  double w[6];
};

// (a, a, b) and its two other permutations, as tri_permutations(5) lists them
// (Quadrature.F90:1821-1826), or the centroid (tri_permutations(4)).
void tri_add_gen(TriRule& r, double a, double w, bool centroid) {
  if (centroid) {
    r.l[r.ngi][0] = r.l[r.ngi][1] = r.l[r.ngi][2] = a;
    r.w[r.ngi++] = w;
    return;
  }
  const double b = 1.0 - 2.0 * a;
  const double c[2] = {a, b};
  const int perm[3][3] = {{1, 1, 2}, {1, 2, 1}, {2, 1, 1}};
  for (int k = 0; k < 3; ++k) {
    for (int j = 0; j < 3; ++j) r.l[r.ngi][j] = c[perm[k][j] - 1];
    r.w[r.ngi++] = w;
  }
}

bool tri_rule(int degree, TriRule& r) {
  r.ngi = 0;
  switch (degree) {
    case 1:
      tri_add_gen(r, 0.333333333333333333333333333333333, 0.5, true);
      return true;
    case 2:
      tri_add_gen(r, 0.166666666666666666666666666666666, 0.166666666666666666666666666666666, false);
      return true;
    case 3:
      tri_add_gen(r, 0.333333333333333333333333333333333, -0.28125, true);
      tri_add_gen(r, 0.2, 0.260416666666666666666666666666666, false);
      return true;
    case 4:
      tri_add_gen(r, 0.0915762135097707434595714634022015, 0.0549758718276609338191631624501052, false);
      tri_add_gen(r, 0.445948490915964886318329253883051, 0.111690794839005732847503504216561, false);
      return true;
    default:
      return false;
  }
}

// Lagrange shape functions on the triangle from barycentric counts.
void tri_shape(int degree, const double l[3], double* n) {
  if (degree == 1) {
    for (int i = 0; i < 3; ++i) n[i] = l[i];
    return;
  }
  const int cnt[6][3] = {{2, 0, 0}, {1, 1, 0}, {0, 2, 0}, {1, 0, 1}, {0, 1, 1}, {0, 0, 2}};
  for (int i = 0; i < 6; ++i) {
    double v = 1.0;
    for (int j = 0; j < 3; ++j) {
      if (cnt[i][j] == 2) v *= l[j] * (2.0 * l[j] - 1.0);
      else if (cnt[i][j] == 1) v *= 2.0 * l[j];
    }
    n[i] = v;
  }
}

}  // namespace

int orc_assemble_advdif_faces(const OrcAdvDifParams* P, int nf, int floc, const int* faces, const int* xfaces,
                              const int* face_ele, const int* ndglno_x, const double* coords,
                              const double* velocity, const double* T, const int* bc_type, const double* bc1,
                              const double* bc2, const int64_t* findrm, const int* colm, double* val,
                              double* rhs) {
  const bool adv = P->have_advection && P->by_parts;
  if (!(adv || P->have_diffusivity)) return ORC_OK;  // (:608-611)
  if (floc != 3 && floc != 6) return ORC_ERR_ARG;
  TriRule q;
  if (!tri_rule(P->quad_degree, q)) return ORC_ERR_ARG;
  const int tdeg = floc == 3 ? 1 : 2;
  double N[6][6], Nu[6][3];  // [gi][node]
  for (int gi = 0; gi < q.ngi; ++gi) {
    tri_shape(tdeg, q.l[gi], N[gi]);
    tri_shape(1, q.l[gi], Nu[gi]);
  }
  const double dt_theta = P->dt * P->theta;
  const double eps0 = 2.220446049250313e-16;
  for (int f = 0; f < nf; ++f) {
    const int ty = bc_type ? bc_type[f] : 0;
    if (ty == 3) continue;
    if (ty != 0 && ty != 1 && ty != 2 && ty != 4) return ORC_ERR_ARG;
    // FLExit: weak Dirichlet with diffusivity (:1371-1375)
    if (ty == 2 && P->have_diffusivity) return ORC_ERR_ARG;
    const int* fn = faces + (int64_t)floc * f;
    const int* xf = xfaces + 3 * (int64_t)f;
    double Xf[3][3];
    for (int j = 0; j < 3; ++j)
      for (int a = 0; a < 3; ++a) Xf[j][a] = coords[3 * (int64_t)xf[j] + a];
    const bool need_t = adv || (P->have_diffusivity && (ty == 1 || ty == 4));
    double detwei[6] = {}, normal[3] = {};
    if (need_t) {
      double J[3][2];
      for (int a = 0; a < 3; ++a) {
        J[a][0] = Xf[0][a] - Xf[2][a];
        J[a][1] = Xf[1][a] - Xf[2][a];
      }
      double detJ = 0.0;
      for (int i = 1; i <= 3; ++i) {
        const int c2 = (i + 1) % 3, c1 = i % 3;  // cyc3(i+2) - 1, cyc3(i+1) - 1
        const double v = J[c2][0] * J[c1][1] - J[c2][1] * J[c1][0];
        detJ += v * v;
      }
      detJ = std::sqrt(detJ);
      for (int gi = 0; gi < q.ngi; ++gi) detwei[gi] = detJ * q.w[gi];
      if (adv) {
        double ow[3], cf[3] = {}, ce[3] = {};
        for (int j = 0; j < 3; ++j)
          for (int a = 0; a < 3; ++a) cf[a] += Xf[j][a];
        const int* ev = ndglno_x + 4 * (int64_t)face_ele[f];
        for (int j = 0; j < 4; ++j)
          for (int a = 0; a < 3; ++a) ce[a] += coords[3 * (int64_t)ev[j] + a];
        for (int a = 0; a < 3; ++a) ow[a] = cf[a] / 3.0 - ce[a] / 4.0;
        double n[3] = {J[1][0] * J[2][1] - J[2][0] * J[1][1], J[2][0] * J[0][1] - J[0][0] * J[2][1],
                       J[0][0] * J[1][1] - J[1][0] * J[0][1]};
        const double o = n[0] * ow[0] + n[1] * ow[1] + n[2] * ow[2];
        for (int a = 0; a < 3; ++a) n[a] *= o;
        const double len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int a = 0; a < 3; ++a) normal[a] = n[a] / len;
      }
    }
    double Tf[6];
    for (int i = 0; i < floc; ++i) Tf[i] = T ? T[fn[i]] : 0.0;
    double Madd[6][6] = {}, Radd[6] = {};
    auto shape_shape = [&](const double* w, double (*out)[6]) {
      for (int i = 0; i < floc; ++i)
        for (int j = 0; j < floc; ++j) {
          double s = 0.0;
          for (int gi = 0; gi < q.ngi; ++gi) s += (N[gi][i] * N[gi][j]) * w[gi];
          out[i][j] = s;
        }
    };
    if (adv) {
      // add_advection_face_cg: u at quad (face_val_at_quad of the P1 velocity)
      double w[6], A[6][6];
      for (int gi = 0; gi < q.ngi; ++gi) {
        double un = 0.0;
        for (int a = 0; a < 3; ++a) {
          double u = 0.0;
          for (int k = 0; k < 3; ++k) u += velocity[3 * (int64_t)xf[k] + a] * Nu[gi][k];
          un += u * normal[a];
        }
        w[gi] = detwei[gi] * un;
      }
      shape_shape(w, A);
      if (std::fabs(dt_theta) > eps0) {
        if (ty == 2) {
          const double* g = bc1 + (int64_t)floc * f;
          for (int i = 0; i < floc; ++i) {
            double s = 0.0;
            for (int j = 0; j < floc; ++j) s += A[i][j] * (g[j] - Tf[j]);
            Radd[i] = Radd[i] - P->theta * s;
          }
        } else {
          for (int i = 0; i < floc; ++i)
            for (int j = 0; j < floc; ++j) Madd[i][j] = Madd[i][j] + dt_theta * A[i][j];
        }
      }
      for (int i = 0; i < floc; ++i) {
        double s = 0.0;
        for (int j = 0; j < floc; ++j) s += A[i][j] * Tf[j];
        Radd[i] = Radd[i] - s;
      }
    }
    if (P->have_diffusivity && (ty == 1 || ty == 4)) {
      // add_diffusivity_face_cg: shape_rhs(N, detwei * g_q) (FETools.F90:38)
      const double* g = bc1 + (int64_t)floc * f;
      double gq[6];
      for (int gi = 0; gi < q.ngi; ++gi) {
        double v = 0.0;
        for (int k = 0; k < floc; ++k) v += g[k] * N[gi][k];
        gq[gi] = detwei[gi] * v;
      }
      for (int i = 0; i < floc; ++i) {
        double s = 0.0;
        for (int gi = 0; gi < q.ngi; ++gi) s += N[gi][i] * gq[gi];
        Radd[i] = Radd[i] + s;
      }
      if (ty == 4) {
        const double* g2 = bc2 + (int64_t)floc * f;
        double w[6], Rm[6][6];
        for (int gi = 0; gi < q.ngi; ++gi) {
          double v = 0.0;
          for (int k = 0; k < floc; ++k) v += g2[k] * N[gi][k];
          w[gi] = detwei[gi] * v;
        }
        shape_shape(w, Rm);
        if (std::fabs(dt_theta) > eps0)
          for (int i = 0; i < floc; ++i)
            for (int j = 0; j < floc; ++j) Madd[i][j] = Madd[i][j] + dt_theta * Rm[i][j];
        for (int i = 0; i < floc; ++i) {
          double s = 0.0;
          for (int j = 0; j < floc; ++j) s += Rm[i][j] * Tf[j];
          Radd[i] = Radd[i] - s;
        }
      }
    }
    // addto(matrix, face_nodes, face_nodes, matrix_addto); addto(rhs, ...)
    for (int i = 0; i < floc; ++i) {
      for (int j = 0; j < floc; ++j) {
        if (Madd[i][j] == 0.0) continue;
        const int64_t p = csr_pos(findrm, colm, fn[i], fn[j]);
        if (p < 0) return ORC_ERR_OUTSIDE_PATTERN;
        val[p] += Madd[i][j];
      }
      rhs[fn[i]] += Radd[i];
    }
  }
  return ORC_OK;
}

// Strong Dirichlet in acceleration form (Boundary_Conditions.F90:1983-2025):
// rows become inactive (Sparse_Tools.F90:2136-2147) and rhs(b) = (g - T)/dt,
// or rhs(b) = g when dt <= 0 is passed (the reference's "no dt" form).
int orc_apply_dirichlet(int nb, const int* nodes, const double* g, const double* T,
                        double dt, double* rhs, unsigned char* inactive) {
  for (int k = 0; k < nb; ++k) {
    int i = nodes[k];
    inactive[i] = 1;
    rhs[i] = dt > 0 ? (g[k] - (T ? T[i] : 0.0)) / dt : g[k];
  }
  return ORC_OK;
}

// ---------------------------------------------------------------------------
// petsc_solve on a csr_matrix with inactive rows (Solvers.F90:111-187,
// 629-921, 1052-1126, 1156-1302; Petsc_Tools.F90:140-298, 891-1060, 671-749):
//  * ghost (inactive) rows are masked out of the PETSc numbering;
//  * rhs lifting b = rhs - A*(rhs on ghost nodes) (Solvers.F90:1072-1104);
//  * ghost columns are dropped and ghost rows carry only the diagonal
//    ghost_pivot = sqrt((max|diag|+min|diag|)*max|diag|/2)
//    (Petsc_Tools.F90:960-985, 1046-1056);
//  * after the solve ghost nodes take their rhs value (Petsc_Tools.F90:726-730).
// The Krylov methods restate PETSc's KSPCG and KSPGMRES (left Jacobi
// preconditioning, preconditioned residual norm, KSPConvergedDefault), the
// third-party library the reference calls at Solvers.F90:1251.
// ---------------------------------------------------------------------------
namespace {

struct Sys {
  int n;
  const int64_t* findrm;
  const int* colm;
  const double* val;
  const unsigned char* ghost;  // may be null
  double pivot;
};

void spmv(const Sys& S, const double* x, double* y) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < S.n; ++i) {
    if (S.ghost && S.ghost[i]) { y[i] = S.pivot * x[i]; continue; }
    double s = 0.0;
    for (int64_t k = S.findrm[i]; k < S.findrm[i + 1]; ++k) {
      int j = S.colm[k];
      if (S.ghost && S.ghost[j]) continue;
      s += S.val[k] * x[j];
    }
    y[i] = s;
  }
}

double dot(int n, const double* a, const double* b) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
  for (int i = 0; i < n; ++i) s += a[i] * b[i];
  return s;
}

struct Conv {
  double rtol, atol, dtol, rnorm0 = 0, ttol = 0;
  int max_its;
  bool guess_zero;
};

// KSPConvergedDefault: returns reason (0 = continue).
int converged(Conv& C, int it, double rnorm, double snorm_b) {
  if (it == 0) {
    if (!C.guess_zero) {
      double snorm = snorm_b;
      if (snorm == 0.0) snorm = rnorm;
      C.rnorm0 = snorm;
    } else {
      C.rnorm0 = rnorm;
    }
    C.ttol = std::max(C.rtol * C.rnorm0, C.atol);
  }
  if (rnorm != rnorm) return -9;  // KSP_DIVERGED_NANORINF
  if (rnorm <= C.ttol) return rnorm < C.atol ? 3 : 2;  // CONVERGED_ATOL / _RTOL
  if (rnorm >= C.dtol * C.rnorm0) return -4;           // DIVERGED_DTOL
  return 0;
}

}  // namespace

int orc_petsc_solve(int n, const int64_t* findrm, const int* colm, const double* val,
                    const unsigned char* inactive, const double* rhs, double* x,
                    int ksp_type /*0 cg, 1 gmres*/, int restart, double rtol, double atol,
                    double dtol, int max_its, int start_from_zero, int* its_out,
                    int* reason_out, double* final_rnorm, double* history, int hist_cap,
                    int nthreads, int norm_type) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  bool any_ghost = false;
  if (inactive)
    for (int i = 0; i < n; ++i) any_ghost = any_ghost || inactive[i];
  Sys S{n, findrm, colm, val, any_ghost ? inactive : nullptr, 0.0};
  // ghost pivot over all rows' |diag| (Petsc_Tools.F90:972-983)
  if (any_ghost) {
    double mind = HUGE_VAL, maxd = -HUGE_VAL;
    for (int i = 0; i < n; ++i) {
      double d = 0.0;
      for (int64_t k = findrm[i]; k < findrm[i + 1]; ++k)
        if (colm[k] == i) d = std::fabs(val[k]);
      mind = std::min(mind, d);
      maxd = std::max(maxd, d);
    }
    S.pivot = std::sqrt((maxd + mind) * maxd / 2.0);
  }
  std::vector<double> b(n), diag(n), y(n, 0.0);
  // rhs lifting of ghost columns (Solvers.F90:1072-1104)
  if (any_ghost) {
    std::vector<double> gh(n), tmp(n);
    for (int i = 0; i < n; ++i) gh[i] = inactive[i] ? rhs[i] : 0.0;
    Sys full{n, findrm, colm, val, nullptr, 0.0};
    spmv(full, gh.data(), tmp.data());
    for (int i = 0; i < n; ++i) b[i] = inactive[i] ? 0.0 : rhs[i] - tmp[i];
  } else {
    for (int i = 0; i < n; ++i) b[i] = rhs[i];
  }
  for (int i = 0; i < n; ++i) {
    if (S.ghost && S.ghost[i]) { diag[i] = S.pivot; continue; }
    double d = 0.0;
    for (int64_t k = findrm[i]; k < findrm[i + 1]; ++k)
      if (colm[k] == i) d = val[k];
    diag[i] = d;
  }
  bool guess_zero = start_from_zero != 0;
  if (!guess_zero)
    for (int i = 0; i < n; ++i) y[i] = (S.ghost && S.ghost[i]) ? 0.0 : x[i];
  // PCJACOBI: B = diag^-1 (a zero diagonal entry is replaced by 1, as PETSc's
  // PCSetUp_Jacobi does).
  std::vector<double> dinv(n);
  for (int i = 0; i < n; ++i) dinv[i] = diag[i] != 0.0 ? 1.0 / diag[i] : 1.0;
  auto pc = [&](const double* r, double* z) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) z[i] = r[i] * dinv[i];
  };
  Conv C{rtol, atol, dtol, 0, 0, max_its, guess_zero};
  // KSPSetNormType: the preconditioned norm ||B r|| (PETSc's default for CG
  // and left-preconditioned GMRES) or, for CG, the unpreconditioned ||r||;
  // the nonzero-guess scale of KSPConvergedDefault is ||B b|| or ||b|| alike.
  const bool unprec = norm_type == 1 && ksp_type == 0;
  std::vector<double> tmpz(n);
  pc(b.data(), tmpz.data());
  double snorm_b = unprec ? std::sqrt(dot(n, b.data(), b.data())) : std::sqrt(dot(n, tmpz.data(), tmpz.data()));
  int nh = 0;
  auto log = [&](double r) { if (history && nh < hist_cap) history[nh] = r; ++nh; };
  int reason = 0, its = 0;
  double rn = 0.0;

  if (ksp_type == 0) {  // KSPCG
    std::vector<double> r(n), z(n), p(n), w(n);
    if (!guess_zero) {
      spmv(S, y.data(), r.data());
      for (int i = 0; i < n; ++i) r[i] = b[i] - r[i];
    } else {
      r = b;
    }
    pc(r.data(), z.data());
    double dp = unprec ? std::sqrt(dot(n, r.data(), r.data())) : std::sqrt(dot(n, z.data(), z.data()));
    rn = dp;
    log(dp);
    reason = converged(C, 0, dp, snorm_b);
    if (!reason) {
      double beta = dot(n, z.data(), r.data()), betaold = 0.0, dpi = 0.0, dpiold = 0.0;
      int i = 0;
      do {
        its = i + 1;
        if (beta == 0.0) { reason = 3; break; }
        if (i > 0 && beta * betaold < 0.0) { reason = -8; break; }
        if (i == 0) {
          p = z;
        } else {
          double bb = beta / betaold;
#pragma omp parallel for schedule(static)
          for (int k = 0; k < n; ++k) p[k] = z[k] + bb * p[k];
        }
        dpiold = dpi;
        spmv(S, p.data(), w.data());
        dpi = dot(n, p.data(), w.data());
        betaold = beta;
        if (dpi == 0.0 || (i > 0 && dpi * dpiold <= 0.0)) { reason = -10; break; }
        double a = beta / dpi;
#pragma omp parallel for schedule(static)
        for (int k = 0; k < n; ++k) {
          y[k] += a * p[k];
          r[k] -= a * w[k];
        }
        pc(r.data(), z.data());
        dp = unprec ? std::sqrt(dot(n, r.data(), r.data())) : std::sqrt(dot(n, z.data(), z.data()));
        rn = dp;
        log(dp);
        reason = converged(C, i + 1, dp, snorm_b);
        if (reason) break;
        beta = dot(n, z.data(), r.data());
        ++i;
      } while (i < max_its);
      if (!reason && i >= max_its) reason = -3;
    }
  } else {  // KSPGMRES, classical Gram-Schmidt, no refinement, haptol 1e-30
    const int m = restart > 0 ? restart : 30;
    std::vector<std::vector<double>> V(m + 1, std::vector<double>(n));
    std::vector<double> H((m + 1) * (m + 1)), cc(m + 1), ss(m + 1), grs(m + 2), nrs(m + 1);
    std::vector<double> t(n), t2(n);
    auto HH = [&](int i, int j) -> double& { return H[(size_t)j * (m + 1) + i]; };
    auto init_resid = [&]() {
      if (guess_zero) {
        pc(b.data(), V[0].data());
      } else {
        spmv(S, y.data(), t.data());
        for (int i = 0; i < n; ++i) t2[i] = b[i] - t[i];
        pc(t2.data(), V[0].data());
      }
    };
    init_resid();
    int itcount = 0;
    bool first = true;
    while (!reason) {
      // KSPGMRESCycle
      // VecNormalize(VEC_VV(0), &res)
      double res = std::sqrt(dot(n, V[0].data(), V[0].data()));
      if (res != 0.0) {
        const double inv = 1.0 / res;
        for (int k = 0; k < n; ++k) V[0][k] *= inv;
      }
      grs[0] = res;
      rn = res;
      int it = 0;
      log(res);
      if (res == 0.0) { reason = 3; }
      else reason = converged(C, its, res, snorm_b);
      (void)first;
      bool hapend = false;
      while (!reason && it < m && its < max_its) {
        spmv(S, V[it].data(), t.data());
        pc(t.data(), V[it + 1].data());
        // classical Gram-Schmidt
        std::vector<double> lhh(it + 1);
        for (int j = 0; j <= it; ++j) lhh[j] = dot(n, V[it + 1].data(), V[j].data());
#pragma omp parallel for schedule(static)
        for (int k = 0; k < n; ++k) {
          double s = V[it + 1][k];
          for (int j = 0; j <= it; ++j) s -= lhh[j] * V[j][k];
          V[it + 1][k] = s;
        }
        for (int j = 0; j <= it; ++j) HH(j, it) = lhh[j];
        double tt = std::sqrt(dot(n, V[it + 1].data(), V[it + 1].data()));
        if (tt != 0.0) {
          double inv = 1.0 / tt;
#pragma omp parallel for schedule(static)
          for (int k = 0; k < n; ++k) V[it + 1][k] *= inv;
        }
        HH(it + 1, it) = tt;
        double hapbnd = std::fabs(tt / grs[it]);
        if (hapbnd > 1e-30) hapbnd = 1e-30;
        if (tt < hapbnd) hapend = true;
        // KSPGMRESUpdateHessenberg
        for (int j = 1; j <= it; ++j) {
          double h0 = HH(j - 1, it), h1 = HH(j, it);
          HH(j - 1, it) = cc[j - 1] * h0 + ss[j - 1] * h1;
          HH(j, it) = cc[j - 1] * h1 - ss[j - 1] * h0;
        }
        if (!hapend) {
          double h0 = HH(it, it), h1 = HH(it + 1, it);
          double r = std::sqrt(h0 * h0 + h1 * h1);
          if (r == 0.0) { reason = -2; break; }
          cc[it] = h0 / r;
          ss[it] = h1 / r;
          grs[it + 1] = -(ss[it] * grs[it]);
          grs[it] = cc[it] * grs[it];
          HH(it, it) = cc[it] * h0 + ss[it] * h1;
          res = std::fabs(grs[it + 1]);
        } else {
          res = 0.0;
        }
        ++it;
        ++its;
        rn = res;
        log(res);
        reason = converged(C, its, res, snorm_b);
        if (hapend && !reason) { reason = -5; break; }
      }
      // KSPGMRESBuildSoln
      int last = it - 1;
      if (last >= 0) {
        nrs[last] = HH(last, last) != 0.0 ? grs[last] / HH(last, last) : 0.0;
        for (int ii = 1; ii <= last; ++ii) {
          int k = last - ii;
          double tt = grs[k];
          for (int j = k + 1; j <= last; ++j) tt -= HH(k, j) * nrs[j];
          nrs[k] = HH(k, k) != 0.0 ? tt / HH(k, k) : 0.0;
        }
#pragma omp parallel for schedule(static)
        for (int k = 0; k < n; ++k) {
          double s = 0.0;
          for (int j = 0; j <= last; ++j) s += nrs[j] * V[j][k];
          y[k] += s;
        }
      }
      itcount += it;
      if (its >= max_its) {
        if (!reason) reason = -3;
        break;
      }
      if (reason) break;
      guess_zero = false;
      init_resid();
      first = false;
    }
  }
  // copy back; ghost nodes take the rhs value (Petsc_Tools.F90:726-730)
  for (int i = 0; i < n; ++i) x[i] = (S.ghost && S.ghost[i]) ? rhs[i] : y[i];
  *its_out = its;
  *reason_out = reason;
  *final_rnorm = rn;
  return nh;
}

// y = A x over the full CSR (csr_mult, Sparse_Tools.F90:3822).
void orc_csr_mult(int n, const int64_t* findrm, const int* colm, const double* val,
                  const double* x, double* y) {
  Sys S{n, findrm, colm, val, nullptr, 0.0};
  spmv(S, x, y);
}

}  // extern "C"

// ===========================================================================
// Pressure projection pieces on a P1 mesh (P1 velocity, P1 pressure).
// ===========================================================================
namespace {

// Triangle rule of degree 2 (Quadrature.F90:936-949, construct_tri_quadratures:
// Str71 three points, permutation 5 (Quadrature.F90:1821-1826) of the
// coordinates (1/6, 1 - 2/6), weight 1/6 each).  Face node i has shape
// function L_i; the P1 face element's dn is d(L1, L2, L3)/d(L1, L2).
struct TriQuad {
  int ngi = 3;
  double l[3][3];
  double w[3];
};
TriQuad tri_quad2() {
  TriQuad t;
  const double c1 = 0.166666666666666666666666666666666, c2 = 1.0 - 2.0 * c1;
  const int perm[3][3] = {{1, 1, 2}, {1, 2, 1}, {2, 1, 1}};
  const double c[2] = {c1, c2};
  for (int k = 0; k < 3; ++k) {
    for (int j = 0; j < 3; ++j) t.l[k][j] = c[perm[k][j] - 1];
    t.w[k] = 0.166666666666666666666666666666666;
  }
  return t;
}

void element_dshape(const double* coords, const int* xn, const Shape& s, int ngi, const Quad& q,
                    double (*dt)[16][3], double* detwei, double* detJ) {
  double X[12];
  for (int i = 0; i < 4; ++i)
    for (int a = 0; a < 3; ++a) X[3 * i + a] = coords[3 * (int64_t)xn[i] + a];
  Geo g;
  element_geometry(X, s, g);
  for (int gi = 0; gi < ngi; ++gi) detwei[gi] = std::fabs(g.detJ) * q.w[gi];
  for (int gi = 0; gi < ngi; ++gi)
    for (int i = 0; i < s.loc; ++i)
      for (int a = 0; a < 3; ++a) {
        double v = 0.0;
        for (int b = 0; b < 3; ++b) v += s.dn[i][gi][b] * g.invJ[a][b];
        dt[i][gi][a] = v;
      }
  if (detJ) *detJ = g.detJ;
}

// solve (femtools/Vector_tools.F90, LAPACK dgesv): Gaussian elimination with
// partial pivoting on the largest magnitude in the column.
void solve_dense(int n, double* A /*row-major n x n*/, double* x) {
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(A[r * n + c]) > std::fabs(A[piv * n + c])) piv = r;
    if (piv != c) {
      for (int k = 0; k < n; ++k) std::swap(A[c * n + k], A[piv * n + k]);
      std::swap(x[c], x[piv]);
    }
    for (int r = c + 1; r < n; ++r) {
      const double f = A[r * n + c] / A[c * n + c];
      for (int k = c; k < n; ++k) A[r * n + k] -= f * A[c * n + k];
      x[r] -= f * x[c];
    }
  }
  for (int r = n - 1; r >= 0; --r) {
    double v = x[r];
    for (int k = r + 1; k < n; ++k) v -= A[r * n + k] * x[k];
    x[r] = v / A[r * n + r];
  }
}

// simplex_tensor (femtools/Metric_tools.F90:852-941): the metric m whose
// unit ball has every edge of the simplex at unit length, from the dof(dim)
// linear system A(edge, idx(k,l)) = diff(k) diff(l) coeff(k,l), A x = 1.
void simplex_tensor(int dim, const double* X /*dim x (dim+1), column = vertex*/, double* m) {
  const int loc = dim + 1, d = dim * (dim + 1) / 2;
  auto idx = [dim](int i, int j) {  // 1-based as in the reference
    const int k = std::min(i, j), l = std::max(i, j);
    if (k == 1) return l;
    return dim == 3 ? l + k : l + k - 1;
  };
  double A[36] = {}, x[6];
  int n = 0;
  for (int i = 0; i < loc; ++i)
    for (int j = i + 1; j < loc; ++j) {
      double diff[3];
      for (int a = 0; a < dim; ++a) diff[a] = X[dim * j + a] - X[dim * i + a];
      for (int k = 1; k <= dim; ++k)
        for (int l = 1; l <= dim; ++l)
          A[n * d + idx(k, l) - 1] = diff[k - 1] * diff[l - 1] * (k == l ? 1.0 : 2.0);
      ++n;
    }
  for (int k = 0; k < d; ++k) x[k] = 1.0;
  solve_dense(d, A, x);
  for (int i = 1; i <= dim; ++i)
    for (int j = 1; j <= dim; ++j) m[(i - 1) * dim + (j - 1)] = x[idx(i, j) - 1];
}

// eigendecomposition_symmetric (femtools/Vector_tools.F90, LAPACK dsyev),
// restated as the cyclic Jacobi method: m = V diag(e) V^T.
void eigen_sym(int n, const double* m, double* V, double* e) {
  double a[9];
  std::memcpy(a, m, sizeof(double) * n * n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) V[i * n + j] = i == j ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) off += a[p * n + q] * a[p * n + q];
    if (off == 0.0) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = a[p * n + q];
        if (apq == 0.0) continue;
        const double th = (a[q * n + q] - a[p * n + p]) / (2.0 * apq);
        const double t = (th >= 0.0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = a[k * n + p], akq = a[k * n + q];
          a[k * n + p] = c * akp - s * akq;
          a[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = a[p * n + k], aqk = a[q * n + k];
          a[p * n + k] = c * apk - s * aqk;
          a[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = V[k * n + p], vkq = V[k * n + q];
          V[k * n + p] = c * vkp - s * vkq;
          V[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < n; ++i) e[i] = a[i * n + i];
}

// edge_length_from_eigenvalue_metric (femtools/Metric_tools.F90:157-164):
// eigenvalues replaced by 1/sqrt(|lambda|) (:145-155) and recomposed.
void edge_length_metric(int n, const double* m, double* out) {
  double V[9], e[3];
  eigen_sym(n, m, V, e);
  for (int i = 0; i < n; ++i) e[i] = 1.0 / std::sqrt(std::fabs(e[i]));
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      double v = 0.0;
      for (int k = 0; k < n; ++k) v += V[i * n + k] * e[k] * V[j * n + k];
      out[i * n + j] = v;
    }
}

// mult_div_invscalar_div_T (femtools/Sparse_Matrices_Fields.F90:673-748):
// product(i,j) = sum_k A(i,k) B(j,k) / s(k) by a merge walk of the sorted
// rows; the output position only advances for entries with a common column.
void mult_div_invscalar(int n, const int64_t* af, const int* ac, const double* av, const double* s,
                        const int64_t* bf, const int* bc, const double* bv, const int64_t* pf,
                        const int* pc, double* out) {
  int64_t nentry0 = 0;
  for (int i = 0; i < n; ++i) {
    const int64_t rb = af[i], re = af[i + 1];
    if (re - rb <= 0) continue;
    for (int64_t jc = pf[i]; jc < pf[i + 1]; ++jc) {
      const int j = pc[jc];
      const int64_t cb = bf[j], ce = bf[j + 1];
      if (ce - cb <= 0) continue;
      double entry0 = 0.0;
      bool addflag = false;
      int64_t k1 = rb, k2 = cb;
      while (k1 < re && k2 < ce) {
        if (ac[k1] < bc[k2]) {
          ++k1;
        } else if (ac[k1] == bc[k2]) {
          entry0 = entry0 + av[k1] * bv[k2] / s[ac[k1]];
          addflag = true;
          ++k1;
          ++k2;
        } else {
          ++k2;
        }
      }
      if (addflag) out[nentry0++] = entry0;
    }
  }
}

}  // namespace

extern "C" {

// compute_lumped_mass (femtools/FEFields.F90:161-214) with unit density:
// row sums of shape_shape(N, N, detwei) added per element.
int orc_lumped_mass(int E, int degree, const int* ndglno, const int* ndglno_x, const double* coords,
                    int quad_degree, int N, double* out) {
  Quad q;
  if (!make_tet_quad(quad_degree, q) || degree < 1 || degree > 2) return ORC_ERR_ARG;
  Shape s, xs;
  make_shape(degree, q, s);
  make_shape(1, q, xs);
  std::memset(out, 0, sizeof(double) * N);
  for (int e = 0; e < E; ++e) {
    double X[12];
    for (int i = 0; i < 4; ++i)
      for (int a = 0; a < 3; ++a) X[3 * i + a] = coords[3 * (int64_t)ndglno_x[4 * (int64_t)e + i] + a];
    Geo g;
    element_geometry(X, xs, g);
    double detwei[16];
    for (int gi = 0; gi < q.ngi; ++gi) detwei[gi] = std::fabs(g.detJ) * q.w[gi];
    const int* nd = ndglno + (int64_t)s.loc * e;
    for (int i = 0; i < s.loc; ++i) {
      double row = 0.0;
      for (int j = 0; j < s.loc; ++j) {
        double m = 0.0;
        for (int gi = 0; gi < q.ngi; ++gi) m += s.n[i][gi] * s.n[j][gi] * detwei[gi];
        row += m;
      }
      out[nd[i]] += row;
    }
  }
  return ORC_OK;
}

// assemble_divergence_matrix_cg (assemble/Divergence_Matrix_CG.F90:67-375)
// for P1 pressure and P1 velocity on one mesh, single phase:
//   not by parts: ele_mat = shape_dshape(N_p, dN_u, detwei)  (FETools.F90:332)
//   by parts:     ele_mat = -dshape_shape(dN_p, N_u, detwei) (FETools.F90:364)
// added per dimension into the blocks ct(dim) over the first-order pattern,
// with the lumped div/grad masses (row sums of shape_shape).  By parts, the
// surface loop (:312-366) adds shape_shape_vector(N, N, detwei_f, normal)
// (FETools.F90:228) into ct(dim) for faces without a boundary condition in
// that dimension (type 0), into ct_rhs against the weak-Dirichlet values
// (type 1) or, for prescribed normal flow (type 5 in dimension 1), subtracts
// shape_rhs(N, detwei_f * g) from ct_rhs; faces of types 2-4 are skipped.
// The face normal is facet_normal (Transform_elements.F90:1527-1553): the
// cross product of the face Jacobian's columns oriented along (face centroid
// - element centroid) and normalised.  bc_type is [face][dim], bc_val is
// [face][face node][dim].  ct holds the three blocks one after the other.
int orc_assemble_divergence_p1(int E, const int* ndglno, const double* coords, int N, const int64_t* findrm,
                               const int* colm, int quad_degree, int by_parts, int nf, const int* faces,
                               const int* face_ele, const int* bc_type, const double* bc_val, double* ct,
                               double* ct_rhs, double* div_ml, double* grad_ml) {
  Quad q;
  if (!make_tet_quad(quad_degree, q)) return ORC_ERR_ARG;
  Shape s;
  make_shape(1, q, s);
  const int64_t nnz = findrm[N] - findrm[0];
  std::memset(ct, 0, sizeof(double) * 3 * nnz);
  if (ct_rhs) std::memset(ct_rhs, 0, sizeof(double) * N);
  if (div_ml) std::memset(div_ml, 0, sizeof(double) * N);
  if (grad_ml) std::memset(grad_ml, 0, sizeof(double) * N);
  for (int e = 0; e < E; ++e) {
    const int* nd = ndglno + 4 * (int64_t)e;
    double dt[10][16][3], detwei[16];
    element_dshape(coords, nd, s, q.ngi, q, dt, detwei, nullptr);
    for (int d = 0; d < 3; ++d)
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
          double v = 0.0;
          for (int gi = 0; gi < q.ngi; ++gi)
            v += detwei[gi] * (by_parts ? dt[i][gi][d] * s.n[j][gi] : s.n[i][gi] * dt[j][gi][d]);
          if (by_parts) v = -v;
          const int64_t p = csr_pos(findrm, colm, nd[i], nd[j]);
          if (p < 0) return ORC_ERR_OUTSIDE_PATTERN;
          ct[d * nnz + p] += v;
        }
    for (int i = 0; i < 4; ++i) {
      double row = 0.0;
      for (int j = 0; j < 4; ++j) {
        double m = 0.0;
        for (int gi = 0; gi < q.ngi; ++gi) m += s.n[i][gi] * s.n[j][gi] * detwei[gi];
        row += m;
      }
      if (div_ml) div_ml[nd[i]] += row;
      if (grad_ml) grad_ml[nd[i]] += row;
    }
  }
  if (!by_parts) return ORC_OK;
  const TriQuad t = tri_quad2();
  for (int f = 0; f < nf; ++f) {
    const int* ty = bc_type + 3 * f;
    bool skip = false;
    for (int d = 0; d < 3; ++d) skip = skip || ty[d] == 2 || ty[d] == 3 || ty[d] == 4;
    if (skip) continue;
    const int* fn = faces + 3 * f;
    const int* en = ndglno + 4 * (int64_t)face_ele[f];
    double Xf[3][3], cf[3] = {0, 0, 0}, ce[3] = {0, 0, 0};
    for (int i = 0; i < 3; ++i)
      for (int a = 0; a < 3; ++a) {
        Xf[i][a] = coords[3 * (int64_t)fn[i] + a];
        cf[a] += Xf[i][a];
      }
    for (int i = 0; i < 4; ++i)
      for (int a = 0; a < 3; ++a) ce[a] += coords[3 * (int64_t)en[i] + a];
    double J[3][2], outward[3];
    for (int a = 0; a < 3; ++a) {
      J[a][0] = Xf[0][a] - Xf[2][a];
      J[a][1] = Xf[1][a] - Xf[2][a];
      outward[a] = cf[a] / 3.0 - ce[a] / 4.0;
    }
    double detJ = 0.0;
    for (int i = 0; i < 3; ++i) {
      const double c = J[cyc3[i + 2]][0] * J[cyc3[i + 1]][1] - J[cyc3[i + 2]][1] * J[cyc3[i + 1]][0];
      detJ += c * c;
    }
    detJ = std::sqrt(detJ);
    double nrm[3] = {J[1][0] * J[2][1] - J[2][0] * J[1][1], J[2][0] * J[0][1] - J[0][0] * J[2][1],
                     J[0][0] * J[1][1] - J[1][0] * J[0][1]};
    const double o = nrm[0] * outward[0] + nrm[1] * outward[1] + nrm[2] * outward[2];
    for (int a = 0; a < 3; ++a) nrm[a] *= o;
    const double len = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    for (int a = 0; a < 3; ++a) nrm[a] /= len;
    double dw[3];
    for (int gi = 0; gi < 3; ++gi) dw[gi] = detJ * t.w[gi];
    const double* bv = bc_val ? bc_val + 9 * f : nullptr;
    if (ty[0] == 5 && ct_rhs) {
      for (int i = 0; i < 3; ++i) {
        double r = 0.0;
        for (int gi = 0; gi < 3; ++gi) {
          double gq = 0.0;
          for (int j = 0; j < 3; ++j) gq += bv[3 * j + 0] * t.l[gi][j];
          r += t.l[gi][i] * (dw[gi] * gq);
        }
        ct_rhs[fn[i]] -= r;
      }
      continue;
    }
    for (int d = 0; d < 3; ++d)
      for (int i = 0; i < 3; ++i) {
        double mrow[3];
        for (int j = 0; j < 3; ++j) {
          double v = 0.0;
          for (int gi = 0; gi < 3; ++gi) v += nrm[d] * (t.l[gi][i] * t.l[gi][j]) * dw[gi];
          mrow[j] = v;
        }
        if (ty[d] == 1 && ct_rhs) {
          double r = 0.0;
          for (int j = 0; j < 3; ++j) r += mrow[j] * bv[3 * j + d];
          ct_rhs[fn[i]] -= r;
        } else {
          for (int j = 0; j < 3; ++j) {
            const int64_t p = csr_pos(findrm, colm, fn[i], fn[j]);
            if (p < 0) return ORC_ERR_OUTSIDE_PATTERN;
            ct[d * nnz + p] += mrow[j];
          }
        }
      }
  }
  return ORC_OK;
}

// make_sparsity(rowmesh, colmesh) (femtools/Sparsity_Patterns.F90:47-85 ->
// make_sparsity_lists :299-379) for two meshes on the same elements: row node
// i of the row mesh holds every column-mesh node of the elements containing
// i, ascending.  The pattern of ct_m (pressure rows, velocity columns).
// Two-call protocol as orc_make_sparsity.
int64_t orc_make_sparsity_rect(int nrows, int E, int loc_r, const int* nd_r, int loc_c, const int* nd_c,
                               int64_t* findrm, int* colm, int64_t cap) {
  std::vector<std::vector<int>> rows(nrows);
  for (int e = 0; e < E; ++e) {
    const int* er = nd_r + (int64_t)loc_r * e;
    const int* ec = nd_c + (int64_t)loc_c * e;
    for (int i = 0; i < loc_r; ++i) {
      std::vector<int>& r = rows[er[i]];
      for (int j = 0; j < loc_c; ++j) {
        auto it = std::lower_bound(r.begin(), r.end(), ec[j]);
        if (it == r.end() || *it != ec[j]) r.insert(it, ec[j]);
      }
    }
  }
  int64_t nnz = 0;
  for (int i = 0; i < nrows; ++i) nnz += (int64_t)rows[i].size();
  if (!colm || cap < nnz) return nnz;
  int64_t p = 0;
  for (int i = 0; i < nrows; ++i) {
    findrm[i] = p;
    for (int c : rows[i]) colm[p++] = c;
  }
  findrm[nrows] = p;
  return nnz;
}

// assemble_divergence_matrix_cg (assemble/Divergence_Matrix_CG.F90:67-375)
// for P1 pressure and P2 velocity (Taylor-Hood) on one affine mesh, single
// phase, the element terms:
//   not by parts: ele_mat(d, i, j) = shape_dshape(N_p, dN_u, detwei)   (FETools.F90:332)
//   by parts:     ele_mat(d, i, j) = -dshape_shape(dN_p, N_u, detwei)  (FETools.F90:364)
// with i over the 4 pressure nodes and j over the 10 velocity nodes, added
// into the blocks ct(d) on the pattern of orc_make_sparsity_rect(p, u).  The
// pressure nodes are the coordinate mesh's vertices (ndglno_p indexes
// coords).  The surface terms of the by-parts form are not restated here.
int orc_assemble_divergence_p2p1(int E, const int* ndglno_p, const int* ndglno_u, const double* coords, int Np,
                                 const int64_t* findrm, const int* colm, int quad_degree, int by_parts,
                                 double* ct) {
  Quad q;
  if (!make_tet_quad(quad_degree, q)) return ORC_ERR_ARG;
  Shape ps, us;
  make_shape(1, q, ps);
  make_shape(2, q, us);
  const int64_t nnz = findrm[Np] - findrm[0];
  std::memset(ct, 0, sizeof(double) * 3 * nnz);
  for (int e = 0; e < E; ++e) {
    const int* pn = ndglno_p + 4 * (int64_t)e;
    const int* un = ndglno_u + 10 * (int64_t)e;
    double X[12];
    for (int i = 0; i < 4; ++i)
      for (int a = 0; a < 3; ++a) X[3 * i + a] = coords[3 * (int64_t)pn[i] + a];
    Geo g;
    element_geometry(X, ps, g);
    double detwei[16];
    for (int gi = 0; gi < q.ngi; ++gi) detwei[gi] = std::fabs(g.detJ) * q.w[gi];
    // physical derivatives of both bases at the quadrature points
    double dp[4][16][3], du[10][16][3];
    for (int gi = 0; gi < q.ngi; ++gi)
      for (int a = 0; a < 3; ++a) {
        for (int i = 0; i < 4; ++i) {
          double v = 0.0;
          for (int b = 0; b < 3; ++b) v += ps.dn[i][gi][b] * g.invJ[a][b];
          dp[i][gi][a] = v;
        }
        for (int j = 0; j < 10; ++j) {
          double v = 0.0;
          for (int b = 0; b < 3; ++b) v += us.dn[j][gi][b] * g.invJ[a][b];
          du[j][gi][a] = v;
        }
      }
    for (int d = 0; d < 3; ++d)
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 10; ++j) {
          double v = 0.0;
          for (int gi = 0; gi < q.ngi; ++gi)
            v += detwei[gi] * (by_parts ? dp[i][gi][d] * us.n[j][gi] : ps.n[i][gi] * du[j][gi][d]);
          if (by_parts) v = -v;
          const int64_t p = csr_pos(findrm, colm, pn[i], un[j]);
          if (p < 0) return ORC_ERR_OUTSIDE_PATTERN;
          ct[d * nnz + p] += v;
        }
  }
  return ORC_OK;
}

// The by-parts surface loop of assemble_divergence_matrix_cg (assemble/
// Divergence_Matrix_CG.F90:312-366) for P1 pressure (test) and P2 velocity
// (field) faces: faces whose bc types include 2, 3 or 4 are skipped; type 5
// in dimension 1 (prescribed normal flow) subtracts shape_rhs(N_p, detwei *
// g) from ct_rhs, g the first component of the velocity bc interpolated with
// the P2 face functions; otherwise ele_mat_bdy = shape_shape_vector(N_p, N_u,
// detwei, normal) (FETools.F90:228) goes, per dimension, into ct_rhs against
// the weak-Dirichlet values (type 1) or into ct_m.  Face transform and
// normal as in orc_assemble_divergence_p1; the triangle rule of quad_degree.
// pfaces: 3 pressure (vertex) nodes per face; ufaces: the 6 velocity nodes
// in the P2 triangle's local order; bc_type [face][dim]; bc_val [face][velocity
// face node][dim].  Adds to ct (the three blocks over the rectangular
// pattern) and ct_rhs (may be null).
int orc_assemble_divergence_p2p1_faces(int nf, const int* pfaces, const int* ufaces, const int* face_ele,
                                       const int* ndglno_x, const double* coords, int Np, const int64_t* findrm,
                                       const int* colm, int quad_degree, const int* bc_type,
                                       const double* bc_val, double* ct, double* ct_rhs) {
  TriRule t;
  if (!tri_rule(quad_degree, t)) return ORC_ERR_ARG;
  double Np_[6][3], Nu[6][6];  // [gi][node]
  for (int gi = 0; gi < t.ngi; ++gi) {
    tri_shape(1, t.l[gi], Np_[gi]);
    tri_shape(2, t.l[gi], Nu[gi]);
  }
  const int64_t nnz = findrm[Np] - findrm[0];
  for (int f = 0; f < nf; ++f) {
    const int* ty = bc_type + 3 * (int64_t)f;
    bool skip = false;
    for (int d = 0; d < 3; ++d) skip = skip || ty[d] == 2 || ty[d] == 3 || ty[d] == 4;
    if (skip) continue;
    const int* fp = pfaces + 3 * (int64_t)f;
    const int* fu = ufaces + 6 * (int64_t)f;
    double Xf[3][3], cf[3] = {0, 0, 0}, ce[3] = {0, 0, 0};
    for (int i = 0; i < 3; ++i)
      for (int a = 0; a < 3; ++a) {
        Xf[i][a] = coords[3 * (int64_t)fp[i] + a];
        cf[a] += Xf[i][a];
      }
    const int* en = ndglno_x + 4 * (int64_t)face_ele[f];
    for (int i = 0; i < 4; ++i)
      for (int a = 0; a < 3; ++a) ce[a] += coords[3 * (int64_t)en[i] + a];
    double J[3][2], outward[3];
    for (int a = 0; a < 3; ++a) {
      J[a][0] = Xf[0][a] - Xf[2][a];
      J[a][1] = Xf[1][a] - Xf[2][a];
      outward[a] = cf[a] / 3.0 - ce[a] / 4.0;
    }
    double detJ = 0.0;
    for (int i = 0; i < 3; ++i) {
      const double c = J[cyc3[i + 2]][0] * J[cyc3[i + 1]][1] - J[cyc3[i + 2]][1] * J[cyc3[i + 1]][0];
      detJ += c * c;
    }
    detJ = std::sqrt(detJ);
    double nrm[3] = {J[1][0] * J[2][1] - J[2][0] * J[1][1], J[2][0] * J[0][1] - J[0][0] * J[2][1],
                     J[0][0] * J[1][1] - J[1][0] * J[0][1]};
    const double o = nrm[0] * outward[0] + nrm[1] * outward[1] + nrm[2] * outward[2];
    for (int a = 0; a < 3; ++a) nrm[a] *= o;
    const double len = std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
    for (int a = 0; a < 3; ++a) nrm[a] /= len;
    double dw[6];
    for (int gi = 0; gi < t.ngi; ++gi) dw[gi] = detJ * t.w[gi];
    const double* bv = bc_val ? bc_val + 18 * (int64_t)f : nullptr;
    if (ty[0] == 5 && ct_rhs) {
      if (!bv) return ORC_ERR_ARG;
      for (int i = 0; i < 3; ++i) {
        double r = 0.0;
        for (int gi = 0; gi < t.ngi; ++gi) {
          double g = 0.0;
          for (int j = 0; j < 6; ++j) g += bv[3 * j + 0] * Nu[gi][j];
          r += Np_[gi][i] * (dw[gi] * g);
        }
        ct_rhs[fp[i]] -= r;
      }
      continue;
    }
    for (int d = 0; d < 3; ++d)
      for (int i = 0; i < 3; ++i) {
        double mrow[6];
        for (int j = 0; j < 6; ++j) {
          double v = 0.0;
          for (int gi = 0; gi < t.ngi; ++gi) v += nrm[d] * (Np_[gi][i] * Nu[gi][j]) * dw[gi];
          mrow[j] = v;
        }
        if (ty[d] == 1 && ct_rhs) {
          if (!bv) return ORC_ERR_ARG;
          double r = 0.0;
          for (int j = 0; j < 6; ++j) r += mrow[j] * bv[3 * j + d];
          ct_rhs[fp[i]] -= r;
        } else {
          for (int j = 0; j < 6; ++j) {
            const int64_t p = csr_pos(findrm, colm, fp[i], fu[j]);
            if (p < 0) return ORC_ERR_OUTSIDE_PATTERN;
            ct[d * nnz + p] += mrow[j];
          }
        }
      }
  }
  return ORC_OK;
}

// make_sparsity_transpose (femtools/Sparsity_Patterns.F90:87-148) for one
// mesh: for every node i, every pair (j, k) of the nodes sharing an element
// with i (row i of the first-order pattern) puts k in row j, ascending
// (insert_ascending).  Two-call protocol: with out_colm == nullptr only the
// entry count is returned.
int64_t orc_sparsity_secondorder(int n, const int64_t* findrm, const int* colm, int64_t* out_findrm,
                                 int* out_colm, int64_t cap) {
  std::vector<std::vector<int>> rows(n);
  for (int i = 0; i < n; ++i)
    for (int64_t a = findrm[i]; a < findrm[i + 1]; ++a) {
      std::vector<int>& r = rows[colm[a]];
      for (int64_t b = findrm[i]; b < findrm[i + 1]; ++b) {
        const int k = colm[b];
        auto it = std::lower_bound(r.begin(), r.end(), k);
        if (it == r.end() || *it != k) r.insert(it, k);
      }
    }
  int64_t nnz = 0;
  out_findrm[0] = 0;
  for (int i = 0; i < n; ++i) {
    if (out_colm)
      for (size_t k = 0; k < rows[i].size(); ++k)
        if (nnz + (int64_t)k < cap) out_colm[nnz + k] = rows[i][k];
    nnz += (int64_t)rows[i].size();
    out_findrm[i + 1] = nnz;
  }
  return nnz;
}

// mult_div_vector_div_T (femtools/Sparse_Matrices_Fields.F90:590-671):
// product(i,j) = sum_k sum_dim A_dim(i,k) B_dim(j,k) w(dim,k) by a merge walk
// of the sorted rows, every product entry written in order.  a and b hold
// ndim blocks of values one after the other, both on the pattern (af, ac)
// (ctp_m and ct_m share the divergence sparsity); w is
// vector_field%val(ndim, ncols).
void orc_mult_div_vector_div_T(int n, int ndim, const int64_t* af, const int* ac, const double* a,
                               const double* w, const double* b, const int64_t* pf, const int* pc,
                               double* out) {
  const int64_t* bf = af;
  const int* bc = ac;
  const int64_t annz = af[n] - af[0];
  int64_t nentry0 = 0;
  for (int i = 0; i < n; ++i)
    for (int64_t jc = pf[i]; jc < pf[i + 1]; ++jc) {
      const int j = pc[jc];
      double entry0 = 0.0;
      int64_t k1 = af[i], k2 = bf[j];
      while (k1 < af[i + 1] && k2 < bf[j + 1]) {
        if (ac[k1] < bc[k2]) {
          ++k1;
        } else if (ac[k1] == bc[k2]) {
          for (int d = 0; d < ndim; ++d)
            entry0 = entry0 + a[d * annz + k1] * b[d * annz + k2] * w[(int64_t)ndim * ac[k1] + d];
          ++k1;
          ++k2;
        } else {
          ++k2;
        }
      }
      out[nentry0++] = entry0;
    }
}

void orc_mult_div_invscalar_div_T(int n, const int64_t* af, const int* ac, const double* a, const double* s,
                                  const int64_t* bf, const int* bc, const double* b, const int64_t* pf,
                                  const int* pc, double* out) {
  mult_div_invscalar(n, af, ac, a, s, bf, bc, b, pf, pc, out);
}

// simplex_tensor and its edge-length form for one simplex (the known answers
// of error_measures/tests/test_simplex_tensor.F90 and
// test_simplex_tensor_edgelens.F90 pin them).
void orc_simplex_tensor(int dim, const double* X, double* m) { simplex_tensor(dim, X, m); }
void orc_edge_length_metric(int dim, const double* m, double* out) { edge_length_metric(dim, m, out); }

// assemble_kmk_matrix (assemble/Momentum_CG.F90:2707-2766) on a P1 pressure
// mesh: kt = sum_e 0.5 dshape_tensor_dshape(dp, h_bar, dp, detwei)
// (FETools.F90:668-698) with h_bar = get_edge_lengths of the element
// (error_measures/Edge_lengths.F90:68-79: edge_length_from_eigenvalue of
// simplex_tensor) at every quadrature point, then
// kmk = mult_div_invscalar_div_T(kt, masslump (times theta_pg unless
// |theta_pg - 1| < epsilon), kt) over the second-order pattern.
int orc_assemble_kmk(int E, const int* ndglno, const double* coords, int N, const int64_t* findrm,
                     const int* colm, int quad_degree, double theta_pg, const double* p_masslump,
                     const int64_t* sof, const int* soc, double* kt, double* kmk) {
  Quad q;
  if (!make_tet_quad(quad_degree, q)) return ORC_ERR_ARG;
  Shape s;
  make_shape(1, q, s);
  const int64_t nnz = findrm[N] - findrm[0];
  std::memset(kt, 0, sizeof(double) * nnz);
  for (int e = 0; e < E; ++e) {
    const int* nd = ndglno + 4 * (int64_t)e;
    double dt[10][16][3], detwei[16];
    element_dshape(coords, nd, s, q.ngi, q, dt, detwei, nullptr);
    double X[12], M[9], H[9];
    for (int i = 0; i < 4; ++i)
      for (int a = 0; a < 3; ++a) X[3 * i + a] = coords[3 * (int64_t)nd[i] + a];
    simplex_tensor(3, X, M);
    edge_length_metric(3, M, H);
    double R[4][4] = {};
    for (int gi = 0; gi < q.ngi; ++gi)
      for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) {
          double v[3];
          for (int b = 0; b < 3; ++b) {
            double t = 0.0;
            for (int a = 0; a < 3; ++a) t += dt[i][gi][a] * H[a * 3 + b];
            v[b] = t;
          }
          double dd = 0.0;
          for (int b = 0; b < 3; ++b) dd += v[b] * dt[j][gi][b];
          R[i][j] = R[i][j] + dd * detwei[gi];
        }
    for (int i = 0; i < 4; ++i)
      for (int j = 0; j < 4; ++j) {
        const int64_t p = csr_pos(findrm, colm, nd[i], nd[j]);
        if (p < 0) return ORC_ERR_OUTSIDE_PATTERN;
        kt[p] += 0.5 * R[i][j];
      }
  }
  std::vector<double> sc(p_masslump, p_masslump + N);
  if (!(std::fabs(theta_pg - 1.0) < 2.220446049250313e-16))
    for (int i = 0; i < N; ++i) sc[i] = p_masslump[i] * theta_pg;
  mult_div_invscalar(N, findrm, colm, kt, sc.data(), findrm, colm, kt, sof, soc, kmk);
  return ORC_OK;
}

}  // extern "C"
