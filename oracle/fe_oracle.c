/*
 * fe_oracle.c -- serial CPU restatement of the FinEtools.jl (v8.2.11)
 * finite-element assembly hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU library and the timed CPU
 * baseline.  Nothing in the product library links or calls this file.
 *
 * Every routine follows the loop order of the reference routine it cites
 * (paths relative to the FinEtools.jl project root).  Compile with
 * -O2 -ffp-contract=off -fno-fast-math so that the arithmetic stays a plain
 * IEEE double evaluation of the reference expressions.
 */
#define _POSIX_C_SOURCE 199309L
#include "fe_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static char g_err[256];
const char *orc_last_error(void) { return g_err; }
static void set_err(const char *m) {
  strncpy(g_err, m, sizeof(g_err) - 1);
  g_err[sizeof(g_err) - 1] = 0;
}

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* ------------------------------------------------------------------ */
/* element facts: nodes per element / manifold dimension               */
/* (src/FESetModule.jl: FESetQ4 711, FESetH8 953, FESetH20 1028,        */
/*  FESetT4 1342, FESetT10 1393)                                        */
/* ------------------------------------------------------------------ */
int orc_nodesperelem(int et) {
  switch (et) {
    case ORC_Q4: return 4;
    case ORC_H8: return 8;
    case ORC_H20: return 20;
    case ORC_T4: return 4;
    case ORC_T10: return 10;
    case ORC_L2: return 2;
  }
  return 0;
}
int orc_manifdim(int et) { return et == ORC_L2 ? 1 : (et == ORC_Q4 ? 2 : 3); }

/* ------------------------------------------------------------------ */
/* Integration rules: GaussRule src/IntegRuleModule.jl:193-398         */
/* (literal constants 211-216; tensor order i outer, k inner 378-390), */
/* TetRule 470-516.                                                     */
/* ------------------------------------------------------------------ */
int orc_gauss_rule(int dim, int order, double *pc, double *w) {
  double x[3], wt[3];
  int n = order;
  if (order == 1) {
    x[0] = 0.0; wt[0] = 2.0;
  } else if (order == 2) {
    x[0] = -0.577350269189626; x[1] = 0.577350269189626;
    wt[0] = 1.0; wt[1] = 1.0;
  } else if (order == 3) {
    x[0] = -0.774596669241483; x[1] = 0.0; x[2] = 0.774596669241483;
    wt[0] = 0.5555555555555556; wt[1] = 0.8888888888888889; wt[2] = 0.5555555555555556;
  } else {
    set_err("Gauss rule order not supported by the oracle");
    return -1;
  }
  int r = 0;
  if (dim == 1) {
    for (int i = 0; i < n; ++i) { pc[i] = x[i]; w[i] = wt[i]; }
    return n;
  } else if (dim == 2) {
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        pc[2 * r] = x[i]; pc[2 * r + 1] = x[j];
        w[r] = wt[i] * wt[j];
        ++r;
      }
    return r;
  } else if (dim == 3) {
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j)
        for (int k = 0; k < n; ++k) {
          pc[3 * r] = x[i]; pc[3 * r + 1] = x[j]; pc[3 * r + 2] = x[k];
          w[r] = wt[i] * wt[j] * wt[k];
          ++r;
        }
    return r;
  }
  set_err("Gauss rule dimension must be 1..3");
  return -1;
}

int orc_tet_rule(int npts, double *pc, double *w) {
  if (npts == 1) {
    pc[0] = 0.25; pc[1] = 0.25; pc[2] = 0.25;
    w[0] = 1.0 / 6.0;
    return 1;
  }
  if (npts == 4) {
    const double a = 0.13819660, b = 0.58541020;
    const double p[12] = {a, a, a, b, a, a, a, b, a, a, a, b};
    memcpy(pc, p, sizeof(p));
    for (int i = 0; i < 4; ++i) w[i] = 0.041666666666666666667;
    return 4;
  }
  set_err("Tet rule: only 1 and 4 points are supported by the oracle");
  return -1;
}

/* ------------------------------------------------------------------ */
/* Basis functions and their parametric gradients (dN row-major nne x  */
/* mdim).  Formulas and node orders as in src/FESetModule.jl: Q4       */
/* 713-733, H8 955-992, H20 1030-1179, T4 1344-1364, T10 1395-1427.     */
/* ------------------------------------------------------------------ */
void orc_bfun(int et, const double *p, double *N) {
  if (et == ORC_L2) { /* src/FESetModule.jl:592-594 */
    N[0] = (1.0 - p[0]) / 2.0;
    N[1] = (1.0 + p[0]) / 2.0;
  } else if (et == ORC_Q4) {
    double x = p[0], y = p[1];
    N[0] = 0.25 * (1.0 - x) * (1.0 - y);
    N[1] = 0.25 * (1.0 + x) * (1.0 - y);
    N[2] = 0.25 * (1.0 + x) * (1.0 + y);
    N[3] = 0.25 * (1.0 - x) * (1.0 + y);
  } else if (et == ORC_H8) {
    double mx = 1.0 - p[0], me = 1.0 - p[1], mt = 1.0 - p[2];
    double px = 1.0 + p[0], pe = 1.0 + p[1], pt = 1.0 + p[2];
    N[0] = mx * me * mt / 8.0;
    N[1] = px * me * mt / 8.0;
    N[2] = px * pe * mt / 8.0;
    N[3] = mx * pe * mt / 8.0;
    N[4] = mx * me * pt / 8.0;
    N[5] = px * me * pt / 8.0;
    N[6] = px * pe * pt / 8.0;
    N[7] = mx * pe * pt / 8.0;
  } else if (et == ORC_H20) {
    double x = p[0], y = p[1], z = p[2];
    double xm = -1 + x, ym = -1 + y, zm = -1 + z;
    double xp = 1 + x, yp = 1 + y, zp = 1 + z;
    const double e = 1.0 / 8, q = 1.0 / 4;
    N[0] = e * xm * ym * zm * (2 + x + y + z);
    N[1] = -e * xp * ym * zm * (2 - x + y + z);
    N[2] = e * xp * yp * zm * (2 - x - y + z);
    N[3] = -e * xm * yp * zm * (2 + x - y + z);
    N[4] = e * xm * ym * zp * (-2 - x - y + z);
    N[5] = -e * xp * ym * zp * (-2 + x - y + z);
    N[6] = e * xp * yp * zp * (-2 + x + y + z);
    N[7] = -e * xm * yp * zp * (-2 - x + y + z);
    N[8] = -q * xm * xp * ym * zm;
    N[9] = q * ym * yp * xp * zm;
    N[10] = q * xm * xp * yp * zm;
    N[11] = -q * ym * yp * xm * zm;
    N[12] = q * xm * xp * ym * zp;
    N[13] = -q * ym * yp * xp * zp;
    N[14] = -q * xm * xp * yp * zp;
    N[15] = q * ym * yp * xm * zp;
    N[16] = -q * zm * zp * xm * ym;
    N[17] = q * zm * zp * xp * ym;
    N[18] = -q * zm * zp * xp * yp;
    N[19] = q * zm * zp * xm * yp;
  } else if (et == ORC_T4) {
    N[0] = 1 - p[0] - p[1] - p[2];
    N[1] = p[0];
    N[2] = p[1];
    N[3] = p[2];
  } else if (et == ORC_T10) {
    double r = p[0], s = p[1], t = p[2];
    double u = 1 - r - s - t;
    N[0] = u * (2 * u - 1);
    N[1] = r * (2 * r - 1);
    N[2] = s * (2 * s - 1);
    N[3] = t * (2 * t - 1);
    N[4] = 4 * u * r;
    N[5] = 4 * r * s;
    N[6] = 4 * s * u;
    N[7] = 4 * u * t;
    N[8] = 4 * r * t;
    N[9] = 4 * s * t;
  }
}

void orc_bfundpar(int et, const double *p, double *d) {
  if (et == ORC_L2) { /* src/FESetModule.jl:595 */
    d[0] = -1.0 / 2.0;
    d[1] = 1.0 / 2.0;
  } else if (et == ORC_Q4) {
    double x = p[0], y = p[1];
    d[0] = -(1.0 - y) * 0.25; d[1] = -(1.0 - x) * 0.25;
    d[2] = (1.0 - y) * 0.25;  d[3] = -(1.0 + x) * 0.25;
    d[4] = (1.0 + y) * 0.25;  d[5] = (1.0 + x) * 0.25;
    d[6] = -(1.0 + y) * 0.25; d[7] = (1.0 - x) * 0.25;
  } else if (et == ORC_H8) {
    double mx = 1.0 - p[0], me = 1.0 - p[1], mt = 1.0 - p[2];
    double px = 1.0 + p[0], pe = 1.0 + p[1], pt = 1.0 + p[2];
    const double g[8][3] = {
        {-me * mt, -mx * mt, -mx * me}, {me * mt, -px * mt, -px * me},
        {pe * mt, px * mt, -px * pe},   {-pe * mt, mx * mt, -mx * pe},
        {-me * pt, -mx * pt, mx * me},  {me * pt, -px * pt, px * me},
        {pe * pt, px * pt, px * pe},    {-pe * pt, mx * pt, mx * pe}};
    for (int k = 0; k < 8; ++k)
      for (int c = 0; c < 3; ++c) d[3 * k + c] = g[k][c] / 8.0;
  } else if (et == ORC_H20) {
    double x = p[0], y = p[1], z = p[2];
    double xm = -(-1 + x), ym = -(-1 + y), zm = -(-1 + z);
    double xp = 1 + x, yp = 1 + y, zp = 1 + z;
    double tppp = 2 + x + y + z, tmpp = 2 - x + y + z, tpmp = 2 + x - y + z;
    double tppm = 2 + x + y - z, tmmp = 2 - x - y + z, tpmm = 2 + x - y - z;
    double tmpm = 2 - x + y - z, tmmm = 2 - x - y - z;
    const double e = 1.0 / 8, q = 1.0 / 4;
    double dx[20] = {
        e * ym * zm * tppp - e * xm * ym * zm, -e * ym * zm * tmpp + e * xp * ym * zm,
        -e * yp * zm * tmmp + e * xp * yp * zm, e * yp * zm * tpmp - e * xm * yp * zm,
        e * ym * zp * tppm - e * xm * ym * zp, -e * ym * zp * tmpm + e * xp * ym * zp,
        -e * yp * zp * tmmm + e * xp * yp * zp, e * yp * zp * tpmm - e * xm * yp * zp,
        -q * xp * ym * zm + q * xm * ym * zm, q * ym * yp * zm,
        -q * xp * yp * zm + q * xm * yp * zm, -q * ym * yp * zm,
        -q * xp * ym * zp + q * xm * ym * zp, q * ym * yp * zp,
        -q * xp * yp * zp + q * xm * yp * zp, -q * ym * yp * zp,
        -q * zm * zp * ym, q * zm * zp * ym, q * zm * zp * yp, -q * zm * zp * yp};
    double dy[20] = {
        e * xm * zm * tppp - e * xm * ym * zm, e * xp * zm * tmpp - e * xp * ym * zm,
        -e * xp * zm * tmmp + e * xp * yp * zm, -e * xm * zm * tpmp + e * xm * yp * zm,
        e * xm * zp * tppm - e * xm * ym * zp, e * xp * zp * tmpm - e * xp * ym * zp,
        -e * xp * zp * tmmm + e * xp * yp * zp, -e * xm * zp * tpmm + e * xm * yp * zp,
        -q * xm * xp * zm, -q * xp * yp * zm + q * xp * ym * zm,
        q * xm * xp * zm, -q * xm * yp * zm + q * xm * ym * zm,
        -q * xm * xp * zp, -q * xp * yp * zp + q * xp * ym * zp,
        q * xm * xp * zp, -q * xm * yp * zp + q * xm * ym * zp,
        -q * zm * zp * xm, -q * zm * zp * xp, q * zm * zp * xp, q * zm * zp * xm};
    double dz[20] = {
        e * xm * ym * tppp - e * xm * ym * zm, e * xp * ym * tmpp - e * xp * ym * zm,
        e * xp * yp * tmmp - e * xp * yp * zm, e * xm * yp * tpmp - e * xm * yp * zm,
        -e * xm * ym * tppm + e * xm * ym * zp, -e * xp * ym * tmpm + e * xp * ym * zp,
        -e * xp * yp * tmmm + e * xp * yp * zp, -e * xm * yp * tpmm + e * xm * yp * zp,
        -q * xm * xp * ym, -q * ym * yp * xp, -q * xm * xp * yp, -q * ym * yp * xm,
        q * xm * xp * ym, q * ym * yp * xp, q * xm * xp * yp, q * ym * yp * xm,
        -q * xm * ym * zp + q * xm * ym * zm, -q * xp * ym * zp + q * xp * ym * zm,
        -q * xp * yp * zp + q * xp * yp * zm, -q * xm * yp * zp + q * xm * yp * zm};
    for (int k = 0; k < 20; ++k) {
      d[3 * k] = dx[k]; d[3 * k + 1] = dy[k]; d[3 * k + 2] = dz[k];
    }
  } else if (et == ORC_T4) {
    const double g[12] = {-1.0, -1.0, -1.0, 1.0, 0.0, 0.0,
                          0.0,  1.0,  0.0,  0.0, 0.0, 1.0};
    memcpy(d, g, sizeof(g));
  } else if (et == ORC_T10) {
    double r = p[0], s = p[1], t = p[2];
    double c = -3 + 4 * r + 4 * s + 4 * t;
    double g[10][3] = {{c, c, c},
                       {4 * r - 1, 0, 0},
                       {0, 4 * s - 1, 0},
                       {0, 0, 4 * t - 1},
                       {-8 * r + 4 - 4 * s - 4 * t, -4 * r, -4 * r},
                       {4 * s, 4 * r, 0},
                       {-4 * s, 4 - 4 * r - 8 * s - 4 * t, -4 * s},
                       {-4 * t, -4 * t, -8 * t + 4 - 4 * r - 4 * s},
                       {4 * t, 0, 4 * r},
                       {0, 4 * t, 4 * s}};
    for (int k = 0; k < 10; ++k)
      for (int m = 0; m < 3; ++m) d[3 * k + m] = g[k][m];
  }
}

/* ------------------------------------------------------------------ */
/* Mesh generators                                                     */
/* ------------------------------------------------------------------ */

/* linearspace (src/MeshUtilModule.jl:116-118) is Julia's
 * range(start, stop, length) whose entries are the correctly rounded
 * start + i*(stop-start)/(n-1); evaluated here with one fma-based
 * correction step of the quotient. */
void orc_linearspace(double start, double stop, int64_t n, double *out) {
  if (n == 1) { out[0] = start; return; }
  double span = stop - start;
  for (int64_t i = 0; i < n; ++i) {
    double hi = (double)i * span;
    double lo = fma((double)i, span, -hi);
    double q = hi / (double)(n - 1);
    double r = fma(-q, (double)(n - 1), hi) + lo;
    q = q + r / (double)(n - 1);
    out[i] = start + q;
  }
  out[n - 1] = stop;
}

/* H8blockx (src/MeshHexahedronModule.jl:59-111): nodes x fastest, then y,
 * then z; cells loop i (x) outer, j (y), k (z) innermost. */
void orc_h8blockx(const double *xs, int64_t nx, const double *ys, int64_t ny,
                  const double *zs, int64_t nz, double *xyz, int64_t *conn) {
  int64_t nL = nx - 1, nW = ny - 1, nH = nz - 1, f = 0;
  for (int64_t k = 0; k <= nH; ++k)
    for (int64_t j = 0; j <= nW; ++j)
      for (int64_t i = 0; i <= nL; ++i) {
        xyz[3 * f] = xs[i]; xyz[3 * f + 1] = ys[j]; xyz[3 * f + 2] = zs[k];
        ++f;
      }
  int64_t gc = 0;
  for (int64_t i = 1; i <= nL; ++i)
    for (int64_t j = 1; j <= nW; ++j)
      for (int64_t k = 1; k <= nH; ++k) {
        int64_t b = (k - 1) * ((nL + 1) * (nW + 1)) + (j - 1) * (nL + 1) + i;
        int64_t t = b + (nL + 1) * (nW + 1);
        int64_t *c = conn + 8 * gc;
        c[0] = b; c[1] = b + 1; c[2] = b + (nL + 1) + 1; c[3] = b + (nL + 1);
        c[4] = t; c[5] = t + 1; c[6] = t + (nL + 1) + 1; c[7] = t + (nL + 1);
        ++gc;
      }
}

/* T4blockx with orientation :a (src/MeshTetrahedronModule.jl:81-150): the
 * same node order as H8blockx; six tetrahedra per cell from the local table
 * at 95-96 (identical for both cell parities with :a). */
void orc_t4blockx(const double *xs, int64_t nx, const double *ys, int64_t ny,
                  const double *zs, int64_t nz, double *xyz, int64_t *conn) {
  static const int tab[6][4] = {{1, 8, 5, 6}, {3, 4, 2, 7}, {7, 2, 6, 8},
                                {4, 7, 8, 2}, {2, 1, 6, 8}, {4, 8, 1, 2}};
  int64_t nL = nx - 1, nW = ny - 1, nH = nz - 1, f = 0;
  for (int64_t k = 0; k <= nH; ++k)
    for (int64_t j = 0; j <= nW; ++j)
      for (int64_t i = 0; i <= nL; ++i) {
        xyz[3 * f] = xs[i]; xyz[3 * f + 1] = ys[j]; xyz[3 * f + 2] = zs[k];
        ++f;
      }
  int64_t gc = 0;
  for (int64_t i = 1; i <= nL; ++i)
    for (int64_t j = 1; j <= nW; ++j)
      for (int64_t k = 1; k <= nH; ++k) {
        int64_t b = (k - 1) * ((nL + 1) * (nW + 1)) + (j - 1) * (nL + 1) + i;
        int64_t t = b + (nL + 1) * (nW + 1);
        int64_t nn[8] = {b, b + 1, b + (nL + 1) + 1, b + (nL + 1),
                         t, t + 1, t + (nL + 1) + 1, t + (nL + 1)};
        for (int r = 0; r < 6; ++r) {
          for (int c = 0; c < 4; ++c) conn[4 * gc + c] = nn[tab[r][c] - 1];
          ++gc;
        }
      }
}

/* Q4blockx (src/MeshQuadrilateralModule.jl:171-214). */
void orc_q4blockx(const double *xs, int64_t nx, const double *ys, int64_t ny,
                  double *xyz, int64_t *conn) {
  int64_t nL = nx - 1, nW = ny - 1, f = 0;
  for (int64_t j = 0; j <= nW; ++j)
    for (int64_t i = 0; i <= nL; ++i) {
      xyz[2 * f] = xs[i]; xyz[2 * f + 1] = ys[j];
      ++f;
    }
  int64_t k = 0;
  for (int64_t i = 1; i <= nL; ++i)
    for (int64_t j = 1; j <= nW; ++j) {
      int64_t b = (j - 1) * (nL + 1) + i;
      conn[4 * k] = b; conn[4 * k + 1] = b + 1;
      conn[4 * k + 2] = b + (nL + 1) + 1; conn[4 * k + 3] = b + (nL + 1);
      ++k;
    }
}

/* H8toH20 (src/MeshHexahedronModule.jl:580-627) and T4toT10
 * (src/MeshTetrahedronModule.jl:158-211): mid-edge nodes are numbered after
 * the existing nodes in first-encounter order (element order x local edge
 * order), keyed by the sorted edge (addhyperface!/findhyperface!,
 * src/MeshUtilModule.jl:41-80), and placed at the mean of the two ends. */
typedef struct { int64_t other, newn, next; } orc_edge;

int64_t orc_quadratic_upgrade(int etype_from, int64_t nelem, const int64_t *conn,
                              int64_t nnodes, const double *xyz,
                              double *xyz_out, int64_t *conn_out) {
  static const int h20e[12][2] = {{1, 2}, {2, 3}, {3, 4}, {4, 1}, {5, 6}, {6, 7},
                                  {7, 8}, {8, 5}, {1, 5}, {2, 6}, {3, 7}, {4, 8}};
  static const int t10e[6][2] = {{1, 2}, {2, 3}, {3, 1}, {4, 1}, {4, 2}, {4, 3}};
  int nv = etype_from == ORC_H8 ? 8 : 4;
  int ne = etype_from == ORC_H8 ? 12 : 6;
  const int(*ec)[2] = etype_from == ORC_H8 ? h20e : t10e;
  int64_t *head = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nnodes + 1));
  orc_edge *pool = (orc_edge *)malloc(sizeof(orc_edge) * (size_t)(nelem * ne + 1));
  for (int64_t i = 0; i <= nnodes; ++i) head[i] = -1;
  int64_t npool = 0, newn = nnodes + 1;
  memcpy(xyz_out, xyz, sizeof(double) * 3 * (size_t)nnodes);
  for (int64_t e = 0; e < nelem; ++e) {
    const int64_t *c = conn + nv * e;
    int64_t *co = conn_out + (nv + ne) * e;
    for (int a = 0; a < nv; ++a) co[a] = c[a];
    for (int J = 0; J < ne; ++J) {
      int64_t n1 = c[ec[J][0] - 1], n2 = c[ec[J][1] - 1];
      int64_t anchor = n1 < n2 ? n1 : n2, other = n1 < n2 ? n2 : n1;
      int64_t found = 0;
      for (int64_t q = head[anchor]; q >= 0; q = pool[q].next)
        if (pool[q].other == other) { found = pool[q].newn; break; }
      if (!found) {
        /* append at the end of the anchor's list (push! order) */
        pool[npool].other = other; pool[npool].newn = newn; pool[npool].next = -1;
        if (head[anchor] < 0) head[anchor] = npool;
        else {
          int64_t q = head[anchor];
          while (pool[q].next >= 0) q = pool[q].next;
          pool[q].next = npool;
        }
        ++npool;
        found = newn++;
        for (int d = 0; d < 3; ++d)
          xyz_out[3 * (found - 1) + d] =
              (xyz[3 * (other - 1) + d] + xyz[3 * (anchor - 1) + d]) * 0.5;
      }
      co[nv + J] = found;
    }
  }
  free(head);
  free(pool);
  return newn - 1;
}

/* ------------------------------------------------------------------ */
/* Node -> element map (src/FENodeToFEMapModule.jl:44-74) and greedy   */
/* colouring element_coloring! (src/MeshModificationModule.jl:1329-1365)*/
/* ------------------------------------------------------------------ */
static void make_n2e(int64_t nelem, int nne, const int64_t *conn, int64_t nnodes,
                     int64_t **ptr_out, int64_t **idx_out) {
  int64_t *ptr = (int64_t *)calloc((size_t)nnodes + 1, sizeof(int64_t));
  for (int64_t e = 0; e < nelem; ++e)
    for (int a = 0; a < nne; ++a) ptr[conn[nne * e + a]]++;
  for (int64_t n = 1; n <= nnodes; ++n) ptr[n] += ptr[n - 1];
  int64_t *idx = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nelem * nne + 1));
  int64_t *fill = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nnodes + 1));
  for (int64_t n = 0; n < nnodes; ++n) fill[n] = ptr[n];
  for (int64_t e = 0; e < nelem; ++e)
    for (int a = 0; a < nne; ++a) {
      int64_t n = conn[nne * e + a] - 1;
      idx[fill[n]++] = e;
    }
  free(fill);
  *ptr_out = ptr;
  *idx_out = idx;
}

int64_t orc_element_coloring(int64_t nelem, int nne, const int64_t *conn,
                             int64_t nnodes, int64_t *colors) {
  int64_t *ptr, *idx;
  make_n2e(nelem, nne, conn, nnodes, &ptr, &idx);
  int64_t cap = 64, ncol = 1;
  int64_t *counts = (int64_t *)calloc((size_t)cap, sizeof(int64_t));
  int64_t *used = (int64_t *)calloc((size_t)cap, sizeof(int64_t));
  for (int64_t e = 0; e < nelem; ++e) colors[e] = 0;
  for (int64_t e = 0; e < nelem; ++e) {
    for (int64_t c = 0; c < ncol; ++c) used[c] = 0;
    int64_t total = 0;
    for (int a = 0; a < nne; ++a) {
      int64_t n = conn[nne * e + a] - 1;
      for (int64_t q = ptr[n]; q < ptr[n + 1]; ++q) {
        int64_t c = colors[idx[q]];
        if (c > 0) { used[c - 1]++; total++; }
      }
    }
    int64_t pick;
    if (total == 0) {
      pick = 0; /* argmin(color_counts): first minimum */
      for (int64_t c = 1; c < ncol; ++c)
        if (counts[c] < counts[pick]) pick = c;
    } else {
      int64_t firstzero = -1;
      for (int64_t c = 0; c < ncol; ++c)
        if (used[c] == 0) { firstzero = c; break; }
      if (firstzero < 0) {
        if (ncol == cap) {
          cap *= 2;
          counts = (int64_t *)realloc(counts, sizeof(int64_t) * (size_t)cap);
          used = (int64_t *)realloc(used, sizeof(int64_t) * (size_t)cap);
        }
        counts[ncol] = 0; used[ncol] = 0;
        pick = ncol++;
      } else {
        /* __find_minimal_count: first unused colour with the smallest count */
        pick = -1;
        int64_t minc = INT64_MAX;
        for (int64_t c = 0; c < ncol; ++c)
          if (used[c] == 0 && minc > counts[c]) { minc = counts[c]; pick = c; }
      }
    }
    colors[e] = pick + 1;
    counts[pick]++;
  }
  free(counts); free(used); free(ptr); free(idx);
  return ncol;
}

int64_t orc_connection_degrees(int64_t nelem, int nne, const int64_t *conn,
                               int64_t nnodes, int64_t *degree) {
  int64_t *ptr, *idx;
  make_n2e(nelem, nne, conn, nnodes, &ptr, &idx);
  int64_t *mark = (int64_t *)malloc(sizeof(int64_t) * (size_t)nnodes);
  for (int64_t n = 0; n < nnodes; ++n) mark[n] = -1;
  int64_t total = 0;
  for (int64_t n = 0; n < nnodes; ++n) {
    int64_t d = 0;
    for (int64_t q = ptr[n]; q < ptr[n + 1]; ++q) {
      const int64_t *c = conn + nne * idx[q];
      for (int a = 0; a < nne; ++a)
        if (mark[c[a] - 1] != n) { mark[c[a] - 1] = n; ++d; }
    }
    degree[n] = d;
    total += d;
  }
  free(mark); free(ptr); free(idx);
  return total;
}

/* ------------------------------------------------------------------ */
/* Sparse matrices: Julia's sparse(I,J,V,m,n) (duplicates combined with */
/* + in input order, rows sorted within columns) and the symmetric     */
/* completion of SysmatAssemblerSparseSymm.makematrix!                  */
/* (src/AssemblyModule.jl:304-329, 551-583).                             */
/* ------------------------------------------------------------------ */
struct orc_matrix {
  int64_t m, n, nnz, zeros_dropped;
  int64_t *colptr, *rowval; /* 1-based */
  double *nzval;
};

int64_t orc_matrix_nnz(const orc_matrix *a) { return a->nnz; }
int64_t orc_matrix_nrows(const orc_matrix *a) { return a->m; }
int64_t orc_matrix_ncols(const orc_matrix *a) { return a->n; }
int64_t orc_matrix_zeros_dropped(const orc_matrix *a) { return a->zeros_dropped; }
void orc_matrix_copy(const orc_matrix *a, int64_t *colptr, int64_t *rowval,
                     double *nzval) {
  memcpy(colptr, a->colptr, sizeof(int64_t) * (size_t)(a->n + 1));
  memcpy(rowval, a->rowval, sizeof(int64_t) * (size_t)a->nnz);
  memcpy(nzval, a->nzval, sizeof(double) * (size_t)a->nnz);
}
void orc_matrix_free(orc_matrix *a) {
  if (!a) return;
  free(a->colptr); free(a->rowval); free(a->nzval); free(a);
}

/* I, J 1-based; consumes nothing; returns a CSC matrix. */
static orc_matrix *sparse_ijv(const int64_t *I, const int64_t *J, const double *V,
                              int64_t len, int64_t m, int64_t n) {
  /* pass 1: counting sort into CSR, keeping input order inside each row */
  int64_t *rp = (int64_t *)calloc((size_t)m + 2, sizeof(int64_t));
  for (int64_t k = 0; k < len; ++k) rp[I[k] + 1]++;
  for (int64_t i = 1; i <= m + 1; ++i) rp[i] += rp[i - 1];
  int64_t *cj = (int64_t *)malloc(sizeof(int64_t) * (size_t)(len + 1));
  double *cv = (double *)malloc(sizeof(double) * (size_t)(len + 1));
  int64_t *pos = (int64_t *)malloc(sizeof(int64_t) * (size_t)(m + 1));
  for (int64_t i = 1; i <= m; ++i) pos[i] = rp[i];
  for (int64_t k = 0; k < len; ++k) {
    int64_t p = pos[I[k]]++;
    cj[p] = J[k];
    cv[p] = V[k];
  }
  /* pass 2: combine duplicates inside each row (left fold in input order) */
  int64_t *last = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n + 1));
  for (int64_t j = 0; j <= n; ++j) last[j] = -1;
  int64_t w = 0;
  int64_t *rp2 = (int64_t *)calloc((size_t)m + 2, sizeof(int64_t));
  for (int64_t i = 1; i <= m; ++i) {
    int64_t start = w;
    rp2[i] = w;
    for (int64_t p = rp[i]; p < rp[i + 1]; ++p) {
      int64_t j = cj[p];
      if (last[j] >= start) {
        cv[last[j]] = cv[last[j]] + cv[p];
      } else {
        last[j] = w;
        cj[w] = j;
        cv[w] = cv[p];
        ++w;
      }
    }
  }
  rp2[m + 1] = w;
  free(last); free(pos); free(rp);
  /* pass 3: transpose CSR -> CSC (rows come out sorted) */
  orc_matrix *A = (orc_matrix *)calloc(1, sizeof(orc_matrix));
  A->m = m; A->n = n; A->nnz = w;
  A->colptr = (int64_t *)calloc((size_t)n + 2, sizeof(int64_t));
  A->rowval = (int64_t *)malloc(sizeof(int64_t) * (size_t)(w + 1));
  A->nzval = (double *)malloc(sizeof(double) * (size_t)(w + 1));
  int64_t *cc = (int64_t *)calloc((size_t)n + 2, sizeof(int64_t));
  for (int64_t p = 0; p < w; ++p) cc[cj[p] + 1]++;
  for (int64_t j = 1; j <= n + 1; ++j) cc[j] += cc[j - 1];
  for (int64_t j = 1; j <= n; ++j) A->colptr[j - 1] = cc[j] + 1;
  A->colptr[n] = w + 1;
  for (int64_t i = 1; i <= m; ++i)
    for (int64_t p = rp2[i]; p < rp2[i + 1]; ++p) {
      int64_t q = cc[cj[p]]++;
      A->rowval[q] = i;
      A->nzval[q] = cv[p];
    }
  free(cc); free(rp2); free(cj); free(cv);
  return A;
}

static orc_matrix *transpose_csc(const orc_matrix *S) {
  orc_matrix *T = (orc_matrix *)calloc(1, sizeof(orc_matrix));
  T->m = S->n; T->n = S->m; T->nnz = S->nnz;
  T->colptr = (int64_t *)calloc((size_t)T->n + 2, sizeof(int64_t));
  T->rowval = (int64_t *)malloc(sizeof(int64_t) * (size_t)(S->nnz + 1));
  T->nzval = (double *)malloc(sizeof(double) * (size_t)(S->nnz + 1));
  int64_t *cc = (int64_t *)calloc((size_t)T->n + 2, sizeof(int64_t));
  for (int64_t p = 0; p < S->nnz; ++p) cc[S->rowval[p]]++;
  int64_t acc = 0;
  for (int64_t j = 1; j <= T->n; ++j) { int64_t t = cc[j]; cc[j] = acc; acc += t; }
  for (int64_t j = 1; j <= T->n; ++j) T->colptr[j - 1] = cc[j] + 1;
  T->colptr[T->n] = S->nnz + 1;
  for (int64_t c = 1; c <= S->n; ++c)
    for (int64_t p = S->colptr[c - 1] - 1; p < S->colptr[c] - 1; ++p) {
      int64_t r = S->rowval[p];
      int64_t q = cc[r]++;
      T->rowval[q] = c;
      T->nzval[q] = S->nzval[p];
    }
  free(cc);
  return T;
}

/* S + transpose(S) with the broadcast rule of SparseArrays' sparse `+`
 * (entries whose sum is exactly zero are not stored), followed by
 * S[j,j] *= 0.5 (a no-op for absent diagonal entries). */
static orc_matrix *symm_complete(orc_matrix *S) {
  orc_matrix *T = transpose_csc(S);
  orc_matrix *C = (orc_matrix *)calloc(1, sizeof(orc_matrix));
  C->m = S->m; C->n = S->n;
  int64_t cap = S->nnz + T->nnz + 1;
  C->colptr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(S->n + 1));
  C->rowval = (int64_t *)malloc(sizeof(int64_t) * (size_t)cap);
  C->nzval = (double *)malloc(sizeof(double) * (size_t)cap);
  int64_t k = 0, dropped = 0;
  for (int64_t j = 1; j <= S->n; ++j) {
    C->colptr[j - 1] = k + 1;
    int64_t a = S->colptr[j - 1] - 1, ae = S->colptr[j] - 1;
    int64_t b = T->colptr[j - 1] - 1, be = T->colptr[j] - 1;
    while (a < ae || b < be) {
      int64_t ra = a < ae ? S->rowval[a] : INT64_MAX;
      int64_t rb = b < be ? T->rowval[b] : INT64_MAX;
      double v;
      int64_t r;
      if (ra == rb) { v = S->nzval[a] + T->nzval[b]; r = ra; ++a; ++b; }
      else if (ra < rb) { v = S->nzval[a] + 0.0; r = ra; ++a; }
      else { v = 0.0 + T->nzval[b]; r = rb; ++b; }
      if (v != 0.0) {
        C->rowval[k] = r;
        C->nzval[k] = (r == j) ? v * 0.5 : v;
        ++k;
      } else {
        ++dropped;
      }
    }
  }
  C->colptr[S->n] = k + 1;
  C->nnz = k;
  C->zeros_dropped = dropped;
  orc_matrix_free(T);
  return C;
}

/* ------------------------------------------------------------------ */
/* COO assemblers (src/AssemblyModule.jl:88-583)                       */
/* ------------------------------------------------------------------ */
struct orc_assembler {
  int kind;
  int64_t nrows, ncols, len, cap;
  int64_t *I, *J;
  double *V;
};

orc_assembler *orc_assembler_create(int kind, int64_t nrows, int64_t ncols) {
  if (kind == ORC_ASM_SPARSE_SYMM && nrows != ncols) {
    set_err("Row and column info do not agree");
    return NULL;
  }
  orc_assembler *a = (orc_assembler *)calloc(1, sizeof(orc_assembler));
  a->kind = kind; a->nrows = nrows; a->ncols = ncols;
  a->cap = 1024;
  a->I = (int64_t *)malloc(sizeof(int64_t) * (size_t)a->cap);
  a->J = (int64_t *)malloc(sizeof(int64_t) * (size_t)a->cap);
  a->V = (double *)malloc(sizeof(double) * (size_t)a->cap);
  return a;
}

static void asm_reserve(orc_assembler *a, int64_t extra) {
  if (a->len + extra <= a->cap) return;
  while (a->len + extra > a->cap) a->cap *= 2;
  a->I = (int64_t *)realloc(a->I, sizeof(int64_t) * (size_t)a->cap);
  a->J = (int64_t *)realloc(a->J, sizeof(int64_t) * (size_t)a->cap);
  a->V = (double *)realloc(a->V, sizeof(double) * (size_t)a->cap);
}

/* assemble! : SysmatAssemblerSparse appends every entry column by column
 * (250-282); SysmatAssemblerSparseSymm appends the lower triangle by local
 * index, i >= j, column by column (500-533).  Same bounds checks. */
int orc_assembler_assemble(orc_assembler *a, const double *mat, int nr, int nc,
                           const int64_t *rows, const int64_t *cols) {
  if (a->kind != ORC_ASM_SPARSE && nr != nc) { set_err("Size mismatch"); return -1; }
  asm_reserve(a, (int64_t)nr * nc);
  if (a->kind == ORC_ASM_DIAG || a->kind == ORC_ASM_HRZ) {
    /* assemble! of the diagonal assemblers (src/AssemblyModule.jl:722-750,
     * 1065-1095): the element matrix's diagonal, for HRZ scaled by the
     * element's total (column sums, then their sum) over its diagonal sum */
    double ffactor = 1.0;
    if (a->kind == ORC_ASM_HRZ) {
      double em2 = 0.0, dem2 = 0.0;
      for (int j = 0; j < nc; ++j) {
        double cs = 0.0;
        for (int i = 0; i < nr; ++i) cs += mat[(size_t)i * nc + j];
        em2 += cs;
      }
      for (int i = 0; i < nr; ++i) dem2 += mat[(size_t)i * nc + i];
      ffactor = em2 / dem2;
    }
    for (int j = 0; j < nc; ++j) {
      int64_t dj = cols[j];
      if (dj < 1) { set_err("Column degree of freedom < 1"); return -1; }
      if (dj > a->ncols) { set_err("Column degree of freedom > size"); return -1; }
      a->I[a->len] = dj;
      a->J[a->len] = dj;
      a->V[a->len] = a->kind == ORC_ASM_HRZ ? mat[(size_t)j * nc + j] * ffactor
                                            : mat[(size_t)j * nc + j];
      a->len++;
    }
    return 0;
  }
  for (int j = 0; j < nc; ++j) {
    int64_t dj = cols[j];
    if (dj < 1) { set_err("Column degree of freedom < 1"); return -1; }
    if (dj > a->ncols) { set_err("Column degree of freedom > size"); return -1; }
    int i0 = a->kind == ORC_ASM_SPARSE_SYMM ? j : 0;
    for (int i = i0; i < nr; ++i) {
      int64_t di = rows[i];
      if (di < 1) { set_err("Row degree of freedom < 1"); return -1; }
      if (di > a->nrows) { set_err("Row degree of freedom > size"); return -1; }
      a->I[a->len] = di;
      a->J[a->len] = dj;
      a->V[a->len] = mat[(size_t)i * nc + j];
      a->len++;
    }
  }
  return 0;
}

static orc_matrix *asm_make_timed(orc_assembler *a, double *t_sparse, double *t_symm) {
  double t0 = now_s();
  orc_matrix *S = sparse_ijv(a->I, a->J, a->V, a->len, a->nrows, a->ncols);
  double t1 = now_s();
  if (t_sparse) *t_sparse = t1 - t0;
  a->len = 0; /* buffer pointer back to 1: ready for the next assembly */
  if (a->kind == ORC_ASM_SPARSE_SYMM) {
    orc_matrix *C = symm_complete(S);
    orc_matrix_free(S);
    if (t_symm) *t_symm = now_s() - t1;
    return C;
  }
  if (t_symm) *t_symm = 0.0;
  return S;
}

orc_matrix *orc_assembler_make(orc_assembler *a) { return asm_make_timed(a, NULL, NULL); }

void orc_assembler_free(orc_assembler *a) {
  if (!a) return;
  free(a->I); free(a->J); free(a->V); free(a);
}

/* ------------------------------------------------------------------ */
/* Element-level kernels                                               */
/* ------------------------------------------------------------------ */

/* locjac! (src/MatrixUtilityModule.jl:60-68): loc = N' X, J = X' dN */
static void locjac(int nne, int sdim, int mdim, const double *X, const double *N,
                   const double *dN, double *loc, double *J) {
  for (int m = 0; m < sdim; ++m) {
    double s = 0.0;
    for (int k = 0; k < nne; ++k) s += N[k] * X[k * sdim + m];
    loc[m] = s;
  }
  for (int n = 0; n < mdim; ++n)
    for (int m = 0; m < sdim; ++m) {
      double s = 0.0;
      for (int k = 0; k < nne; ++k) s += X[k * sdim + m] * dN[k * mdim + n];
      J[m * mdim + n] = s;
    }
}

/* Jacobian (src/FESetModule.jl:387-391 one-manifold, 426-435 two-manifold,
 * 479-489 three-manifold) */
static double jac_det(int sdim, int mdim, const double *J) {
#define JJ(r, c) J[((r) - 1) * mdim + ((c) - 1)]
  if (mdim == 1) {
    double s = 0.0;
    for (int r = 1; r <= sdim; ++r) s += JJ(r, 1) * JJ(r, 1);
    return sqrt(s);
  }
  if (mdim == 3) {
    return JJ(1, 1) * (JJ(2, 2) * JJ(3, 3) - JJ(3, 2) * JJ(2, 3)) -
           JJ(1, 2) * (JJ(2, 1) * JJ(3, 3) - JJ(2, 3) * JJ(3, 1)) +
           JJ(1, 3) * (JJ(2, 1) * JJ(3, 2) - JJ(2, 2) * JJ(3, 1));
  }
  if (sdim == 2) return JJ(1, 1) * JJ(2, 2) - JJ(2, 1) * JJ(1, 2);
  double c1 = JJ(2, 1) * JJ(3, 2) - JJ(3, 1) * JJ(2, 2);
  double c2 = JJ(3, 1) * JJ(1, 2) - JJ(1, 1) * JJ(3, 2);
  double c3 = JJ(1, 1) * JJ(2, 2) - JJ(2, 1) * JJ(1, 2);
  return sqrt(c1 * c1 + c2 * c2 + c3 * c3);
#undef JJ
}

/* gradN! (src/FESetModule.jl:453-470 two-manifold, 507-544 three-manifold);
 * redJ is mdim x mdim. */
static void grad_n(int nne, int mdim, const double *dN, const double *R, double *g) {
#define RR(r, c) R[((r) - 1) * mdim + ((c) - 1)]
  if (mdim == 3) {
    double invdet = 1.0 / (+RR(1, 1) * (RR(2, 2) * RR(3, 3) - RR(3, 2) * RR(2, 3)) -
                           RR(1, 2) * (RR(2, 1) * RR(3, 3) - RR(2, 3) * RR(3, 1)) +
                           RR(1, 3) * (RR(2, 1) * RR(3, 2) - RR(2, 2) * RR(3, 1)));
    double i11 = (RR(2, 2) * RR(3, 3) - RR(3, 2) * RR(2, 3)) * invdet;
    double i12 = -(RR(1, 2) * RR(3, 3) - RR(1, 3) * RR(3, 2)) * invdet;
    double i13 = (RR(1, 2) * RR(2, 3) - RR(1, 3) * RR(2, 2)) * invdet;
    double i21 = -(RR(2, 1) * RR(3, 3) - RR(2, 3) * RR(3, 1)) * invdet;
    double i22 = (RR(1, 1) * RR(3, 3) - RR(1, 3) * RR(3, 1)) * invdet;
    double i23 = -(RR(1, 1) * RR(2, 3) - RR(2, 1) * RR(1, 3)) * invdet;
    double i31 = (RR(2, 1) * RR(3, 2) - RR(3, 1) * RR(2, 2)) * invdet;
    double i32 = -(RR(1, 1) * RR(3, 2) - RR(3, 1) * RR(1, 2)) * invdet;
    double i33 = (RR(1, 1) * RR(2, 2) - RR(2, 1) * RR(1, 2)) * invdet;
    for (int r = 0; r < nne; ++r) {
      const double *d = dN + 3 * r;
      g[3 * r] = d[0] * i11 + d[1] * i21 + d[2] * i31;
      g[3 * r + 1] = d[0] * i12 + d[1] * i22 + d[2] * i32;
      g[3 * r + 2] = d[0] * i13 + d[1] * i23 + d[2] * i33;
    }
  } else {
    double invdet = 1.0 / (RR(1, 1) * RR(2, 2) - RR(1, 2) * RR(2, 1));
    double i11 = (RR(2, 2)) * invdet, i12 = -(RR(1, 2)) * invdet;
    double i21 = -(RR(2, 1)) * invdet, i22 = (RR(1, 1)) * invdet;
    for (int r = 0; r < nne; ++r) {
      const double *d = dN + 2 * r;
      g[2 * r] = d[0] * i11 + d[1] * i21;
      g[2 * r + 1] = d[0] * i12 + d[1] * i22;
    }
  }
#undef RR
}

/* blmat!(DeforModelRed3D) with the identity material frame
 * (src/DeforModelRedModule.jl:447-472); B is 6 x 3nne row-major. */
static void blmat3d(int nne, const double *g, const double *rm, double *B) {
  int n = 3 * nne;
  memset(B, 0, sizeof(double) * 6 * (size_t)n);
  for (int i = 0; i < nne; ++i)
    for (int j = 0; j < 3; ++j) {
      int kj = 3 * i + j;
      /* Rm[j, :] (the identity when no material frame is given) */
      double R1 = rm ? rm[3 * j] : (j == 0), R2 = rm ? rm[3 * j + 1] : (j == 1);
      double R3 = rm ? rm[3 * j + 2] : (j == 2);
      const double *gi = g + 3 * i;
      B[0 * n + kj] = gi[0] * R1;
      B[1 * n + kj] = gi[1] * R2;
      B[2 * n + kj] = gi[2] * R3;
      B[3 * n + kj] = gi[1] * R1 + gi[0] * R2;
      B[4 * n + kj] = gi[2] * R1 + gi[0] * R3;
      B[5 * n + kj] = gi[2] * R2 + gi[1] * R3;
    }
}

static const double *coef_at(const orc_coef *c, int64_t e, int q, int npts) {
  if (c->kind == ORC_COEF_CONST) return c->data;
  if (c->kind == ORC_COEF_PER_ELEMENT) return c->data + (size_t)e * c->ncomp;
  return c->data + ((size_t)e * npts + q) * c->ncomp;
}

static const double kPi = 3.14159265358979323846; /* Julia's pi as Float64 */

/* Jacobianmdim / Jacobianvolume (src/IntegDomainModule.jl:370-383, 405-450,
 * 504-549, 567-602): a two-manifold integrated as a volume, and a curve
 * integrated as a surface or a volume, are scaled by the other dimension;
 * on an axisymmetric domain by 2 pi r instead (r = loc[0]), a curve
 * integrated as a volume by both. */
static double jac_mdim(const orc_problem *p, int mdim, const double *J, const double *loc,
                       int m) {
  double d = jac_det(p->sdim, mdim, J);
  if (mdim == 2 && m == 3) return p->axisymmetric ? d * 2 * kPi * loc[0] : d * p->otherdim;
  if (mdim == 1 && m == 2) return p->axisymmetric ? d * 2 * kPi * loc[0] : d * p->otherdim;
  if (mdim == 1 && m == 3)
    return p->axisymmetric ? d * 2 * kPi * loc[0] * p->otherdim : d * p->otherdim;
  return d;
}

/* Rm' J (mulCAtB!, src/MatrixUtilityModule.jl:478-521) for a 3-manifold in a
 * constant material frame; J itself for the identity frame */
static const double *rmtj(const orc_problem *p, int mdim, const double *J, double *out) {
  if (!p->rm || mdim != 3) return J;
  for (int a = 0; a < 3; ++a)
    for (int b = 0; b < 3; ++b) {
      double s = 0.0;
      for (int k = 0; k < 3; ++k) s += p->rm[k * 3 + a] * J[k * 3 + b];
      out[a * 3 + b] = s;
    }
  return out;
}

orc_matrix *orc_bilform(const orc_problem *p, int form, const orc_coef *c, int m,
                        int asm_kind, double *phase) {
  int nne = orc_nodesperelem(p->etype), mdim = orc_manifdim(p->etype);
  int sdim = p->sdim, ndn = p->ndn, npts = p->npts;
  int n = nne * ndn;
  if (mdim == 3 && m != 3) { set_err("That is the only acceptable option here."); return NULL; }
  if (form == ORC_LIN_ELASTIC && (ndn != 3 || mdim != 3 || sdim != 3 || c->ncomp != 36)) {
    set_err("lin_elastic: 3-D solids, ndn = 3, 6x6 D"); return NULL;
  }
  if (form == ORC_DIFFUSION && !(c->ncomp == 1 || c->ncomp == mdim * mdim)) {
    set_err("diffusion: scalar or mdim x mdim coefficient"); return NULL;
  }
  if (form == ORC_DIFFUSION && mdim != sdim) {
    set_err("diffusion: the manifold must fill the space"); return NULL;
  }
  if (form == ORC_DOT && c->ncomp != ndn * ndn) { set_err("dot: ndn x ndn coefficient"); return NULL; }
  if (form == ORC_DIV_GRAD && (c->ncomp != 1 || ndn != mdim || mdim != sdim)) {
    set_err("div_grad: scalar viscosity, ndn = mdim = sdim"); return NULL;
  }
  double *Ns = (double *)malloc(sizeof(double) * npts * nne);
  double *dNs = (double *)malloc(sizeof(double) * npts * nne * mdim);
  for (int q = 0; q < npts; ++q) {
    if (p->Ns) memcpy(Ns + q * nne, p->Ns + q * nne, sizeof(double) * nne);
    else orc_bfun(p->etype, p->pc + q * mdim, Ns + q * nne);
    if (p->dNs) memcpy(dNs + q * nne * mdim, p->dNs + q * nne * mdim, sizeof(double) * nne * mdim);
    else orc_bfundpar(p->etype, p->pc + q * mdim, dNs + q * nne * mdim);
  }
  double *X = (double *)malloc(sizeof(double) * nne * sdim);
  double *Ke = (double *)malloc(sizeof(double) * n * n);
  double *g = (double *)malloc(sizeof(double) * nne * mdim);
  double *B = (double *)malloc(sizeof(double) * 6 * n);
  double *DB = (double *)malloc(sizeof(double) * 6 * n);
  double *kg = (double *)malloc(sizeof(double) * mdim * nne);
  int64_t *dofs = (int64_t *)malloc(sizeof(int64_t) * n);
  double loc[3], J[9], RmTJ[9];
  orc_assembler *a = orc_assembler_create(asm_kind, p->nalldofs, p->nalldofs);
  if (!a) return NULL;
  asm_reserve(a, p->nelem * (asm_kind == ORC_ASM_SPARSE_SYMM ? (int64_t)(n * n + n) / 2
                                                              : (int64_t)n * n));
  double t0 = now_s();
  int iso = (form == ORC_DIFFUSION && c->ncomp == 1);
  for (int64_t e = 0; e < p->nelem; ++e) {
    const int64_t *ce = p->conn + (size_t)e * nne;
    for (int k = 0; k < nne; ++k)
      for (int d = 0; d < sdim; ++d) X[k * sdim + d] = p->xyz[(size_t)(ce[k] - 1) * sdim + d];
    memset(Ke, 0, sizeof(double) * n * n);
    for (int q = 0; q < npts; ++q) {
      const double *N = Ns + q * nne, *dN = dNs + q * nne * mdim;
      locjac(nne, sdim, mdim, X, N, dN, loc, J);
      const double *cv = coef_at(c, e, q, npts);
      if (form == ORC_DIFFUSION) {
        double Jac = jac_mdim(p, mdim, J, loc, 3);
        if (iso) {
          grad_n(nne, mdim, dN, J, g); /* the iso form ignores the frame */
          /* add_mggt_ut_only! (src/MatrixUtilityModule.jl:84-98) */
          double mult = cv[0] * Jac * p->w[q];
          for (int nx = 0; nx < nne; ++nx)
            for (int px = 0; px < mdim; ++px) {
              double av = mult * g[nx * mdim + px];
              for (int mx = 0; mx <= nx; ++mx) Ke[mx * n + nx] += g[mx * mdim + px] * av;
            }
        } else {
          /* RmTJ = Rm' J (src/FEMMBaseModule.jl:1495-1497), gradients in the
           * material frame */
          grad_n(nne, mdim, dN, rmtj(p, mdim, J, RmTJ), g);
          /* add_gkgt_ut_only! (src/MatrixUtilityModule.jl:120-153) */
          double Jw = Jac * p->w[q];
          for (int nx = 0; nx < nne; ++nx)
            for (int mx = 0; mx < mdim; ++mx) {
              double acc = 0.0;
              for (int px = 0; px < mdim; ++px) acc += cv[mx * mdim + px] * g[nx * mdim + px];
              kg[mx * nne + nx] = Jw * acc;
            }
          for (int nx = 0; nx < nne; ++nx)
            for (int mx = 0; mx <= nx; ++mx) {
              double acc = 0.0;
              for (int px = 0; px < mdim; ++px) acc += g[mx * mdim + px] * kg[px * nne + nx];
              Ke[mx * n + nx] += acc;
            }
        }
      } else if (form == ORC_LIN_ELASTIC) {
        double Jac = jac_mdim(p, mdim, J, loc, 3);
        /* src/FEMMBaseModule.jl:1801-1804: RmTJ = Rm' J, blmat! with Rm */
        grad_n(nne, mdim, dN, rmtj(p, mdim, J, RmTJ), g);
        blmat3d(nne, g, p->rm, B);
        /* add_btdb_ut_only! (src/MatrixUtilityModule.jl:189-216) */
        double Jw = Jac * p->w[q];
        for (int nx = 0; nx < n; ++nx)
          for (int mx = 0; mx < 6; ++mx) {
            double acc = 0.0;
            for (int px = 0; px < 6; ++px) acc += cv[mx * 6 + px] * B[px * n + nx];
            DB[mx * n + nx] = Jw * acc;
          }
        for (int nx = 0; nx < n; ++nx)
          for (int mx = 0; mx <= nx; ++mx) {
            double acc = 0.0;
            for (int px = 0; px < 6; ++px) acc += B[px * n + mx] * DB[px * n + nx];
            Ke[mx * n + nx] += acc;
          }
      } else if (form == ORC_DIV_GRAD) {
        /* bilform_div_grad, src/FEMMBaseModule.jl:1690-1710 (full matrix) */
        double Jac = jac_mdim(p, mdim, J, loc, 3);
        grad_n(nne, mdim, dN, J, g);
        double factor = cv[0] * (Jac * p->w[q]);
        for (int aa = 0; aa < nne; ++aa)
          for (int bb = 0; bb < nne; ++bb)
            for (int s = 0; s < ndn; ++s) {
              int pr = aa * ndn + s, rc = bb * ndn + s;
              for (int qq = 0; qq < ndn; ++qq)
                Ke[pr * n + rc] += factor * g[aa * mdim + qq] * g[bb * mdim + qq];
              for (int qq = 0; qq < ndn; ++qq) {
                rc = bb * ndn + qq;
                Ke[pr * n + rc] += factor * g[aa * mdim + qq] * g[bb * mdim + s];
              }
            }
      } else { /* ORC_DOT, src/FEMMBaseModule.jl:1348-1364 */
        double Jac = jac_mdim(p, mdim, J, loc, m);
        for (int k = 0; k < nne; ++k)
          for (int mm = 0; mm < nne; ++mm) {
            double factor = N[k] * N[mm] * Jac * p->w[q];
            for (int pp = 0; pp < ndn; ++pp)
              for (int qq = 0; qq < ndn; ++qq)
                Ke[(k * ndn + pp) * n + mm * ndn + qq] += factor * cv[pp * ndn + qq];
          }
      }
    }
    if (form != ORC_DOT && form != ORC_DIV_GRAD) /* complete_lt! (src/MatrixUtilityModule.jl:164-173) */
      for (int nx = 0; nx < n; ++nx)
        for (int mx = nx + 1; mx < n; ++mx) Ke[mx * n + nx] = Ke[nx * n + mx];
    /* gatherdofnums! (src/FieldModule.jl:304-314): node-major order */
    for (int k = 0; k < nne; ++k)
      for (int d = 0; d < ndn; ++d) dofs[k * ndn + d] = p->dofnums[(size_t)(ce[k] - 1) * ndn + d];
    if (orc_assembler_assemble(a, Ke, n, n, dofs, dofs) != 0) {
      orc_assembler_free(a);
      return NULL;
    }
  }
  double t1 = now_s();
  double ts = 0, tc = 0;
  orc_matrix *K = asm_make_timed(a, &ts, &tc);
  if (phase) { phase[0] = t1 - t0; phase[1] = ts; phase[2] = tc; }
  orc_assembler_free(a);
  free(Ns); free(dNs); free(X); free(Ke); free(g); free(B); free(DB); free(kg); free(dofs);
  return K;
}

/* bilform_convection (src/FEMMBaseModule.jl:1583-1625) into
 * SysmatAssemblerSparse: K[p, r] += N_p (u . grad N_r) Jac w with u the
 * interpolated velocity (nnodes x nsd, row-major here); the density rhof is
 * evaluated by the reference but does not enter the matrix.  Scalar field. */
orc_matrix *orc_bilform_convection(const orc_problem *p, const double *vel, int nsd) {
  int nne = orc_nodesperelem(p->etype), mdim = orc_manifdim(p->etype);
  int sdim = p->sdim, npts = p->npts;
  if (p->ndn != 1) { set_err("convection: scalar field"); return NULL; }
  if (mdim != sdim || nsd != sdim) { set_err("convection: nsd = sdim = mdim"); return NULL; }
  double *Ns = (double *)malloc(sizeof(double) * npts * nne);
  double *dNs = (double *)malloc(sizeof(double) * npts * nne * mdim);
  for (int q = 0; q < npts; ++q) {
    if (p->Ns) memcpy(Ns + q * nne, p->Ns + q * nne, sizeof(double) * nne);
    else orc_bfun(p->etype, p->pc + q * mdim, Ns + q * nne);
    if (p->dNs) memcpy(dNs + q * nne * mdim, p->dNs + q * nne * mdim, sizeof(double) * nne * mdim);
    else orc_bfundpar(p->etype, p->pc + q * mdim, dNs + q * nne * mdim);
  }
  double *X = (double *)malloc(sizeof(double) * nne * sdim);
  double *U = (double *)malloc(sizeof(double) * nne * nsd);
  double *Ke = (double *)malloc(sizeof(double) * nne * nne);
  double *g = (double *)malloc(sizeof(double) * nne * mdim);
  int64_t *dofs = (int64_t *)malloc(sizeof(int64_t) * nne);
  double loc[3], J[9];
  orc_assembler *a = orc_assembler_create(ORC_ASM_SPARSE, p->nalldofs, p->nalldofs);
  asm_reserve(a, p->nelem * (int64_t)nne * nne);
  for (int64_t e = 0; e < p->nelem; ++e) {
    const int64_t *ce = p->conn + (size_t)e * nne;
    for (int k = 0; k < nne; ++k) {
      for (int d = 0; d < sdim; ++d) X[k * sdim + d] = p->xyz[(size_t)(ce[k] - 1) * sdim + d];
      for (int d = 0; d < nsd; ++d) U[k * nsd + d] = vel[(size_t)(ce[k] - 1) * nsd + d];
    }
    memset(Ke, 0, sizeof(double) * nne * nne);
    for (int q = 0; q < npts; ++q) {
      const double *N = Ns + q * nne, *dN = dNs + q * nne * mdim;
      locjac(nne, sdim, mdim, X, N, dN, loc, J);
      double Jac = jac_mdim(p, mdim, J, loc, 3);
      grad_n(nne, mdim, dN, J, g);
      for (int pp = 0; pp < nne; ++pp)
        for (int r = 0; r < nne; ++r) {
          double accum = 0.0;
          for (int s = 0; s < nsd; ++s) {
            double u_s = 0.0;
            for (int k = 0; k < nne; ++k) u_s += N[k] * U[k * nsd + s];
            accum += u_s * g[r * mdim + s];
          }
          Ke[pp * nne + r] += N[pp] * accum * (Jac * p->w[q]);
        }
    }
    for (int k = 0; k < nne; ++k) dofs[k] = p->dofnums[(size_t)(ce[k] - 1)];
    if (orc_assembler_assemble(a, Ke, nne, nne, dofs, dofs) != 0) {
      orc_assembler_free(a);
      return NULL;
    }
  }
  orc_matrix *K = orc_assembler_make(a);
  orc_assembler_free(a);
  free(Ns); free(dNs); free(X); free(U); free(Ke); free(g); free(dofs);
  return K;
}

/* bilform_masslike (src/FEMMBaseModule.jl:1865-1917) into
 * SysmatAssemblerSparse: a rectangular matrix of nelem*ndn rows (the ndn
 * rows of element i are (i-1)*ndn+1 .. i*ndn) and nalldofs columns; element
 * block M[p, (b-1)*ndn + q] += N_b Jac w c[p, q], Jac = Jacobianmdim(m). */
orc_matrix *orc_bilform_masslike(const orc_problem *p, const orc_coef *c, int m) {
  int nne = orc_nodesperelem(p->etype), mdim = orc_manifdim(p->etype);
  int sdim = p->sdim, ndn = p->ndn, npts = p->npts;
  int nc = nne * ndn;
  if (mdim == 3 && m != 3) { set_err("That is the only acceptable option here."); return NULL; }
  if (c->ncomp != ndn * ndn) { set_err("masslike: ndn x ndn coefficient"); return NULL; }
  double *Ns = (double *)malloc(sizeof(double) * npts * nne);
  double *dNs = (double *)malloc(sizeof(double) * npts * nne * mdim);
  for (int q = 0; q < npts; ++q) {
    if (p->Ns) memcpy(Ns + q * nne, p->Ns + q * nne, sizeof(double) * nne);
    else orc_bfun(p->etype, p->pc + q * mdim, Ns + q * nne);
    if (p->dNs) memcpy(dNs + q * nne * mdim, p->dNs + q * nne * mdim, sizeof(double) * nne * mdim);
    else orc_bfundpar(p->etype, p->pc + q * mdim, dNs + q * nne * mdim);
  }
  double *X = (double *)malloc(sizeof(double) * nne * sdim);
  double *Me = (double *)malloc(sizeof(double) * ndn * nc);
  int64_t *rows = (int64_t *)malloc(sizeof(int64_t) * ndn);
  int64_t *dofs = (int64_t *)malloc(sizeof(int64_t) * nc);
  double loc[3], J[9];
  orc_assembler *a = orc_assembler_create(ORC_ASM_SPARSE, p->nelem * ndn, p->nalldofs);
  if (!a) return NULL;
  asm_reserve(a, p->nelem * (int64_t)ndn * nc);
  for (int64_t e = 0; e < p->nelem; ++e) {
    const int64_t *ce = p->conn + (size_t)e * nne;
    for (int k = 0; k < nne; ++k)
      for (int d = 0; d < sdim; ++d) X[k * sdim + d] = p->xyz[(size_t)(ce[k] - 1) * sdim + d];
    memset(Me, 0, sizeof(double) * ndn * nc);
    for (int q = 0; q < npts; ++q) {
      const double *N = Ns + q * nne, *dN = dNs + q * nne * mdim;
      locjac(nne, sdim, mdim, X, N, dN, loc, J);
      double Jac = jac_mdim(p, mdim, J, loc, m);
      const double *cv = coef_at(c, e, q, npts);
      for (int b = 0; b < nne; ++b) {
        double factor = N[b] * Jac * p->w[q];
        for (int pp = 0; pp < ndn; ++pp)
          for (int qq = 0; qq < ndn; ++qq) Me[pp * nc + b * ndn + qq] += factor * cv[pp * ndn + qq];
      }
    }
    for (int k = 0; k < nne; ++k)
      for (int d = 0; d < ndn; ++d) dofs[k * ndn + d] = p->dofnums[(size_t)(ce[k] - 1) * ndn + d];
    for (int pp = 0; pp < ndn; ++pp) rows[pp] = e * ndn + pp + 1;
    if (orc_assembler_assemble(a, Me, ndn, nc, rows, dofs) != 0) {
      orc_assembler_free(a);
      return NULL;
    }
  }
  orc_matrix *M = orc_assembler_make(a);
  orc_assembler_free(a);
  free(Ns); free(dNs); free(X); free(Me); free(rows); free(dofs);
  return M;
}

/* linform_dot (src/FEMMBaseModule.jl:1207-1244) into SysvecAssembler
 * (src/AssemblyModule.jl:885-917). */
int orc_linform_dot(const orc_problem *p, const orc_coef *f, int m, double *F) {
  int nne = orc_nodesperelem(p->etype), mdim = orc_manifdim(p->etype);
  int sdim = p->sdim, ndn = p->ndn, npts = p->npts;
  if (mdim == 3 && m != 3) { set_err("That is the only acceptable option here."); return -1; }
  if (f->ncomp != ndn) { set_err("force must have ndn components"); return -1; }
  double *Ns = (double *)malloc(sizeof(double) * npts * nne);
  double *dNs = (double *)malloc(sizeof(double) * npts * nne * mdim);
  for (int q = 0; q < npts; ++q) {
    if (p->Ns) memcpy(Ns + q * nne, p->Ns + q * nne, sizeof(double) * nne);
    else orc_bfun(p->etype, p->pc + q * mdim, Ns + q * nne);
    if (p->dNs) memcpy(dNs + q * nne * mdim, p->dNs + q * nne * mdim, sizeof(double) * nne * mdim);
    else orc_bfundpar(p->etype, p->pc + q * mdim, dNs + q * nne * mdim);
  }
  double *X = (double *)malloc(sizeof(double) * nne * sdim);
  double *Fe = (double *)malloc(sizeof(double) * nne * ndn);
  double loc[3], J[9];
  for (int64_t i = 0; i < p->nalldofs; ++i) F[i] = 0.0;
  for (int64_t e = 0; e < p->nelem; ++e) {
    const int64_t *ce = p->conn + (size_t)e * nne;
    for (int k = 0; k < nne; ++k)
      for (int d = 0; d < sdim; ++d) X[k * sdim + d] = p->xyz[(size_t)(ce[k] - 1) * sdim + d];
    for (int r = 0; r < nne * ndn; ++r) Fe[r] = 0.0;
    for (int q = 0; q < npts; ++q) {
      const double *N = Ns + q * nne, *dN = dNs + q * nne * mdim;
      locjac(nne, sdim, mdim, X, N, dN, loc, J);
      double Jac = jac_mdim(p, mdim, J, loc, m);
      const double *force = coef_at(f, e, q, npts);
      double Factor = Jac * p->w[q];
      int rx = 0;
      for (int kx = 0; kx < nne; ++kx) {
        double NkxF = N[kx] * Factor;
        for (int mx = 0; mx < ndn; ++mx) { Fe[rx] = Fe[rx] + NkxF * force[mx]; ++rx; }
      }
    }
    for (int k = 0; k < nne; ++k)
      for (int d = 0; d < ndn; ++d) {
        int64_t gi = p->dofnums[(size_t)(ce[k] - 1) * ndn + d];
        if (gi < 1) { set_err("Row degree of freedom < 1"); return -1; }
        if (gi > p->nalldofs) { set_err("Row degree of freedom > size"); return -1; }
        F[gi - 1] += Fe[k * ndn + d];
      }
  }
  free(Ns); free(dNs); free(X); free(Fe);
  return 0;
}
