// fl_refelem.h -- reference tetrahedron data on the host: quadrature rules
// and Lagrange P1/P2 basis values and derivatives at the quadrature points.
//
// Rules: the symmetric tet rules of femtools/Quadrature.F90:649-735 (degree 1
// Str71 1 point, degree 2 Str71 4 points, degree 3 Str71 5 points, degree 4
// kea86 11 points); a request for degree d takes the lowest rule of degree
// >= d (Quadrature.F90:318).  Points are barycentric (l1..l4); weights sum to
// the reference volume 1/6.
// Basis: local node order of number_tets_lagrange
// (femtools/Element_Numbering.F90:389-472); values N and derivatives with
// respect to l1, l2, l3 with l4 = 1 - l1 - l2 - l3 (diffl4 = -1,
// femtools/Elements.F90:693-717).
#pragma once

#include <cstring>

namespace fl {

struct TetQuad {
  int degree = 0, ngi = 0;
  double l[16][4];
  double w[16];
};

inline void tq_push(TetQuad& q, double w, double a, double b, double c, double d) {
  q.l[q.ngi][0] = a;
  q.l[q.ngi][1] = b;
  q.l[q.ngi][2] = c;
  q.l[q.ngi][3] = d;
  q.w[q.ngi] = w;
  ++q.ngi;
}

// Orbit of (a,a,a,b): the point with b in slot 4, 3, 2, 1 in that order.
inline void tq_orbit4(TetQuad& q, double w, double a, double b) {
  tq_push(q, w, a, a, a, b);
  tq_push(q, w, a, a, b, a);
  tq_push(q, w, a, b, a, a);
  tq_push(q, w, b, a, a, a);
}

// Orbit of (a,a,b,b): six points, b-pairs in slots (3,4),(2,4),(2,3),(1,4),(1,3),(1,2).
inline void tq_orbit6(TetQuad& q, double w, double a, double b) {
  tq_push(q, w, a, a, b, b);
  tq_push(q, w, a, b, a, b);
  tq_push(q, w, a, b, b, a);
  tq_push(q, w, b, a, a, b);
  tq_push(q, w, b, a, b, a);
  tq_push(q, w, b, b, a, a);
}

inline bool tet_quadrature(int degree, TetQuad& q) {
  q = TetQuad();
  if (degree <= 1) {
    tq_push(q, 0.166666666666666666666666666666666, 0.25, 0.25, 0.25, 0.25);
    q.degree = 1;
  } else if (degree == 2) {
    const double a = 0.138196601125010515179541316563436;
    tq_orbit4(q, 0.041666666666666666666666666666666, a, 1.0 - 3.0 * a);
    q.degree = 2;
  } else if (degree == 3) {
    tq_push(q, -0.133333333333333333333333333333333, 0.25, 0.25, 0.25, 0.25);
    const double a = 0.166666666666666666666666666666666;
    tq_orbit4(q, 0.075, a, 1.0 - 3.0 * a);
    q.degree = 3;
  } else if (degree == 4) {
    tq_push(q, -0.013155555555555555555555555555555, 0.25, 0.25, 0.25, 0.25);
    const double a = 0.0714285714285714285714285714285714;
    tq_orbit4(q, 7.62222222222222222222222222222222E-3, a, 1.0 - 3.0 * a);
    const double c = 0.399403576166799204996102147461640;
    tq_orbit6(q, 0.0248888888888888888888888888888888, c, 0.5 - c);
    q.degree = 4;
  } else {
    return false;
  }
  return true;
}

struct TetShape {
  int loc = 0;
  double n[10][16];
  double dn[10][16][3];
};

// Barycentric counts of the local nodes (degree 1: the vertices; degree 2:
// vertex 1, edge 12, vertex 2, edge 13, edge 23, vertex 3, edge 14, edge 24,
// edge 34, vertex 4).
inline int tet_node_counts(int degree, int (*c)[4]) {
  static const int p1[4][4] = {{1, 0, 0, 0}, {0, 1, 0, 0}, {0, 0, 1, 0}, {0, 0, 0, 1}};
  static const int p2[10][4] = {{2, 0, 0, 0}, {1, 1, 0, 0}, {0, 2, 0, 0}, {1, 0, 1, 0}, {0, 1, 1, 0},
                                {0, 0, 2, 0}, {1, 0, 0, 1}, {0, 1, 0, 1}, {0, 0, 1, 1}, {0, 0, 0, 2}};
  if (degree == 1) {
    std::memcpy(c, p1, sizeof(p1));
    return 4;
  }
  std::memcpy(c, p2, sizeof(p2));
  return 10;
}

// 1-D factor of the simplex Lagrange basis for count k at spacing 1/degree,
// normalised to 1 at l = k/degree; value and derivative.
inline void lagrange_factor(int k, int degree, double l, double* v, double* dv) {
  double h = 1.0 / degree, val = 1.0, norm = 1.0, der = 0.0;
  for (int m = 0; m < k; ++m) {
    double prod = 1.0;
    for (int r = 0; r < k; ++r)
      if (r != m) prod *= (l - r * h);
    der += prod;
    val *= (l - m * h);
    norm *= (k * h - m * h);
  }
  *v = val / norm;
  *dv = der / norm;
}

inline void tet_shape(int degree, const TetQuad& q, TetShape& s) {
  int c[10][4];
  s = TetShape();
  s.loc = tet_node_counts(degree, c);
  for (int i = 0; i < s.loc; ++i)
    for (int g = 0; g < q.ngi; ++g) {
      double v[4], dv[4];
      for (int j = 0; j < 4; ++j) lagrange_factor(c[i][j], degree, q.l[g][j], &v[j], &dv[j]);
      s.n[i][g] = v[0] * v[1] * v[2] * v[3];
      for (int d = 0; d < 3; ++d) {
        // d/dl_d of f_d(l_d) f_4(l_4(l_d)) times the other two factors
        double x = dv[d] * v[3] - dv[3] * v[d];
        for (int j = 0; j < 3; ++j)
          if (j != d) x *= v[j];
        s.dn[i][g][d] = x;
      }
    }
}

// Triangle rules of degree 1..4 (Quadrature.F90 construct_tri_quadratures,
// Str71 and the degree-4 six-point rule): (a, a, b) generators expanded in
// the order of tri_permutations(5), or the centroid.
inline int tri_rule(int degree, double l[6][3], double w[6]) {
  int n = 0;
  auto cen = [&](double a, double wt) {
    l[n][0] = l[n][1] = l[n][2] = a;
    w[n++] = wt;
  };
  auto gen = [&](double a, double wt) {
    const double b = 1.0 - 2.0 * a;
    const double c[2] = {a, b};
    const int perm[3][3] = {{1, 1, 2}, {1, 2, 1}, {2, 1, 1}};
    for (int k = 0; k < 3; ++k) {
      for (int j = 0; j < 3; ++j) l[n][j] = c[perm[k][j] - 1];
      w[n++] = wt;
    }
  };
  switch (degree) {
    case 1: cen(0.333333333333333333333333333333333, 0.5); break;
    case 2: gen(0.166666666666666666666666666666666, 0.166666666666666666666666666666666); break;
    case 3:
      cen(0.333333333333333333333333333333333, -0.28125);
      gen(0.2, 0.260416666666666666666666666666666);
      break;
    case 4:
      gen(0.0915762135097707434595714634022015, 0.0549758718276609338191631624501052);
      gen(0.445948490915964886318329253883051, 0.111690794839005732847503504216561);
      break;
    default: return 0;
  }
  return n;
}

// Lagrange functions of a face triangle at barycentric point l, host side
// (P1: the barycentrics; P2: vertex L(2L-1), edge 4 L_a L_b in the local
// order vertex 1, edge 12, vertex 2, edge 13, edge 23, vertex 3).
inline void tri_lagrange(int floc, const double l[3], double* n) {
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

}  // namespace fl
