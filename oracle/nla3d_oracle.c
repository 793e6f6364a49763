/* ORACLE -- test infrastructure, never on the product path.
 *
 * A plain-C restatement of nla3d's per-iteration assembly (reference paths are
 * relative to the reference's src/lib/):
 *   DoF registration / numbering     FEStorage.cpp:338-432, Dof.cpp:33-67
 *   CSR pattern                      FEStorage.cpp:434-550, SparseMatrix.cpp:44-114
 *   value routing / lookup           BlockSparseMatrix.h:126-168, SparseMatrix.cpp:117-154,467-479
 *   hexahedron Jacobian              isoparametric.cpp:140-188, 211-221
 *   hyperelastic S and D             materials_hyperelastic.cpp:30-129, 135-204, solidmech.cpp
 *   SOLID81 update / buildK / scatter SOLID81.cpp:85-191, SOLID81.h:54-94
 *   TETRA0 buildK                    TETRA0.cpp:18-78, 110-199
 *   QUADTH buildK                    QUADTH.cpp:22-49, isoparametric.cpp:55-129
 *   rigid-body MPC rows              Mpc.cpp:52-164, FEStorage.cpp:41-61
 * Every floating-point expression keeps the reference's operand order and
 * association (and the dense zero-padded products of Mat.h), so with
 * -ffp-contract=off the results equal the compiled reference's bit for bit;
 * the tests check exactly that against oracle/_ref and the committed goldens.
 * The dense products are also what the reference spends its time on, which is
 * why this port is a fair stand-in for the reference's CPU timing.
 */
#include "nla3d_oracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define NDOFT 8 /* Dof::numberOfDofTypes (Dof.h:15-25) */
enum { UX = 0, UY, UZ, ROTX, ROTY, ROTZ, HYDRO_PRESSURE, TEMP };
enum { ET_PLANE41 = 1, ET_SOLID81 = 2, ET_TETRA0 = 3, ET_QUADTH = 5 };
enum { MAT_NH = 1, MAT_BID = 2, MAT_MR = 3 };
/* element parameters kept per element: TETRA0 (E, my), QUADTH (k, volFlux,
 * rho, c) (TETRA0.h, QUADTH.h:29-35) */
#define EPAR 4
static const uint32_t INVALID = 0xFFFFFFFFu; /* SparseMatrix.cpp:11 */

/* ----------------------------------------------------------------------- */
/* dense kernels, Mat.h:686-801 (row-major, packed-upper symmetric)         */
/* ----------------------------------------------------------------------- */

static inline __attribute__((always_inline)) void k_matBTDBprod(int M, int N, const double* B, const double* D, double coef, double* R) {
  /* Mat<dimN,dimM> A on the stack, zeroed (Mat.h:689-690) */
  double A[24 * 24];
  if (N * M > 24 * 24) abort();
  memset(A, 0, sizeof(double) * (size_t)N * M);
  const double* Dp = D;
  /* A = B^T * (upper part of D incl. diagonal) */
  for (int k = 0; k < M; k++)
    for (int j = k; j < M; j++) {
      for (int i = 0; i < N; i++) A[i * M + j] += B[k * N + i] * (*Dp);
      Dp++;
    }
  /* A += B^T * (strict upper part of D, transposed) */
  Dp = D;
  for (int j = 0; j < M; j++) {
    Dp++;
    for (int k = j + 1; k < M; k++) {
      for (int i = 0; i < N; i++) A[i * M + j] += B[k * N + i] * (*Dp);
      Dp++;
    }
  }
  double* Rp = R;
  for (int i = 0; i < N; i++)
    for (int j = i; j < N; j++) {
      for (int k = 0; k < M; k++) *Rp += A[i * M + k] * B[k * N + j] * coef;
      Rp++;
    }
}

static inline __attribute__((always_inline)) void k_matBTVprod(int M, int N, const double* B, const double* V, double coef, double* R) {
  for (int i = 0; i < N; i++)
    for (int j = 0; j < M; j++) R[i] += B[j * N + i] * V[j] * coef;
}

static inline __attribute__((always_inline)) void k_matBVprod(int M, int N, const double* B, const double* V, double coef, double* R) {
  for (int i = 0; i < M; i++)
    for (int j = 0; j < N; j++) R[i] += B[i * N + j] * V[j] * coef;
}

static inline __attribute__((always_inline)) void k_matABprod(int M1, int N1, int N2, const double* A, const double* B, double coef,
                   double* R) {
  double* Rp = R;
  for (int i = 0; i < M1; i++)
    for (int j = 0; j < N2; j++) {
      for (int k = 0; k < N1; k++) *Rp += A[i * N1 + k] * B[k * N2 + j] * coef;
      Rp++;
    }
}

static inline __attribute__((always_inline)) void k_matATBprod(int M1, int N1, int N2, const double* A, const double* B, double coef,
                    double* R) {
  double* Rp = R;
  for (int i = 0; i < N1; i++)
    for (int j = 0; j < N2; j++) {
      for (int k = 0; k < M1; k++) *Rp += A[k * N1 + i] * B[k * N2 + j] * coef;
      Rp++;
    }
}

/* exported wrappers (the mat_prod known-answer tests call these) */
void orc_matBTDBprod(int M, int N, const double* B, const double* D, double coef, double* R) {
  k_matBTDBprod(M, N, B, D, coef, R);
}
void orc_matBTVprod(int M, int N, const double* B, const double* V, double coef, double* R) {
  k_matBTVprod(M, N, B, V, coef, R);
}
void orc_matBVprod(int M, int N, const double* B, const double* V, double coef, double* R) {
  k_matBVprod(M, N, B, V, coef, R);
}
void orc_matABprod(int M1, int N1, int N2, const double* A, const double* B, double coef,
                   double* R) {
  k_matABprod(M1, N1, N2, A, B, coef, R);
}
void orc_matATBprod(int M1, int N1, int N2, const double* A, const double* B, double coef,
                    double* R) {
  k_matATBprod(M1, N1, N2, A, B, coef, R);
}

/* Mat<3,3>::det / inv (Mat.cpp:23-46) */
static double det3(const double d[3][3]) {
  return d[0][0] * (d[1][1] * d[2][2] - d[1][2] * d[2][1]) -
         d[0][1] * (d[1][0] * d[2][2] - d[1][2] * d[2][0]) +
         d[0][2] * (d[1][0] * d[2][1] - d[1][1] * d[2][0]);
}

static void inv3(const double d[3][3], double det, double r[3][3]) {
  double t[9] = {d[1][1] * d[2][2] - d[1][2] * d[2][1], d[0][2] * d[2][1] - d[0][1] * d[2][2],
                 d[0][1] * d[1][2] - d[0][2] * d[1][1], d[2][0] * d[1][2] - d[1][0] * d[2][2],
                 d[0][0] * d[2][2] - d[0][2] * d[2][0], d[1][0] * d[0][2] - d[0][0] * d[1][2],
                 d[1][0] * d[2][1] - d[1][1] * d[2][0], d[0][1] * d[2][0] - d[0][0] * d[2][1],
                 d[0][0] * d[1][1] - d[0][1] * d[1][0]};
  const double s = 1.0 / det;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) r[i][j] = t[i * 3 + j] * s;
}

/* ----------------------------------------------------------------------- */
/* isoparametric hexahedron / quad (isoparametric.h:118-192, .cpp:55-221)   */
/* ----------------------------------------------------------------------- */

static const double GP_A = 0.5773502691896258; /* isoparametric.h:127 */
static const double GP_B = 0.7745966692414834; /* isoparametric.h:141 */

typedef struct { double r, s, t, w; } quad3;
typedef struct { double r, s, w; } quad2;

static int hex_rule(int order, quad3* q) {
  if (order <= 1) {
    q[0].r = q[0].s = q[0].t = 0.0;
    q[0].w = 8.0;
    return 1;
  }
  if (order == 2) {
    for (int n = 0; n < 8; n++) {
      q[n].r = (n & 1) ? GP_A : -GP_A;
      q[n].s = (n & 2) ? GP_A : -GP_A;
      q[n].t = (n & 4) ? GP_A : -GP_A;
      q[n].w = 1.0;
    }
    return 8;
  }
  /* 3rd order, r fastest then s then t (isoparametric.h:140-178) */
  static const double pts[3] = {-0.7745966692414834, 0.0, 0.7745966692414834};
  static const double wt3[27] = {
      0.1714677640603567, 0.2743484224965707, 0.1714677640603567, 0.2743484224965707,
      0.4389574759945130, 0.2743484224965707, 0.1714677640603567, 0.2743484224965707,
      0.1714677640603567, 0.2743484224965707, 0.4389574759945130, 0.2743484224965707,
      0.4389574759945130, 0.7023319615912207, 0.4389574759945130, 0.2743484224965707,
      0.4389574759945130, 0.2743484224965707, 0.1714677640603567, 0.2743484224965707,
      0.1714677640603567, 0.2743484224965707, 0.4389574759945130, 0.2743484224965707,
      0.1714677640603567, 0.2743484224965707, 0.1714677640603567};
  (void)GP_B;
  int n = 0;
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++, n++) {
        q[n].r = pts[i];
        q[n].s = pts[j];
        q[n].t = pts[k];
        q[n].w = wt3[n];
      }
  return 27;
}

static void hex_dN(double r, double s, double t, double dN[8][3]) {
  const double v[24] = {
      -0.125 * (1.0 - s) * (1.0 - t), -0.125 * (1.0 - r) * (1.0 - t), -0.125 * (1.0 - r) * (1.0 - s),
      +0.125 * (1.0 - s) * (1.0 - t), -0.125 * (1.0 + r) * (1.0 - t), -0.125 * (1.0 + r) * (1.0 - s),
      +0.125 * (1.0 + s) * (1.0 - t), +0.125 * (1.0 + r) * (1.0 - t), -0.125 * (1.0 + r) * (1.0 + s),
      -0.125 * (1.0 + s) * (1.0 - t), +0.125 * (1.0 - r) * (1.0 - t), -0.125 * (1.0 - r) * (1.0 + s),
      -0.125 * (1.0 - s) * (1.0 + t), -0.125 * (1.0 - r) * (1.0 + t), +0.125 * (1.0 - r) * (1.0 - s),
      +0.125 * (1.0 - s) * (1.0 + t), -0.125 * (1.0 + r) * (1.0 + t), +0.125 * (1.0 + r) * (1.0 - s),
      +0.125 * (1.0 + s) * (1.0 + t), +0.125 * (1.0 + r) * (1.0 + t), +0.125 * (1.0 + r) * (1.0 + s),
      -0.125 * (1.0 + s) * (1.0 + t), +0.125 * (1.0 - r) * (1.0 + t), +0.125 * (1.0 - r) * (1.0 + s)};
  memcpy(dN, v, sizeof(v));
}

/* returns the number of integration points; NiXj is np x 8 x 3 */
static int hex_jacobian(const double X[8][3], int order, double* NiXj, double* det, double* wts) {
  quad3 q[27];
  if (order < 1) order = 1;
  if (order > 3) order = 3;
  const int np = hex_rule(order, q);
  for (int g = 0; g < np; g++) {
    double dN[8][3];
    hex_dN(q[g].r, q[g].s, q[g].t, dN);
    double J[3][3] = {{0}};
    for (int a = 0; a < 8; a++)
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) J[i][j] += dN[a][i] * X[a][j];
    det[g] = det3(J);
    double Ji[3][3];
    inv3(J, det[g], Ji);
    double* G = NiXj + (size_t)g * 24;
    memset(G, 0, sizeof(double) * 24);
    for (int a = 0; a < 8; a++)
      for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) G[a * 3 + i] += Ji[i][j] * dN[a][j];
    if (wts) wts[g] = q[g].w;
  }
  return np;
}

void orc_hex_jacobian(const double* X, int int_order, double* NiXj, double* det) {
  hex_jacobian((const double(*)[3])X, int_order, NiXj, det, NULL);
}

static int quad_jacobian(const double X[4][3], int order, double* NiXj /*np x 4 x 2*/,
                         double* det, double* wts, double* N /*np x 4*/) {
  static const double o3p[3] = {-0.7745966692414834, 0.0, 0.7745966692414834};
  static const double o3w[9] = {0.3086419753086420, 0.4938271604938271, 0.3086419753086420,
                                0.4938271604938271, 0.7901234567901234, 0.4938271604938271,
                                0.3086419753086420, 0.4938271604938271, 0.3086419753086420};
  quad2 q[9];
  int np;
  if (order < 1) order = 1;
  if (order > 3) order = 3;
  if (order == 1) {
    q[0].r = q[0].s = 0.0;
    q[0].w = 4.0;
    np = 1;
  } else if (order == 2) {
    for (int n = 0; n < 4; n++) {
      q[n].r = (n & 1) ? GP_A : -GP_A;
      q[n].s = (n & 2) ? GP_A : -GP_A;
      q[n].w = 1.0;
    }
    np = 4;
  } else {
    np = 0;
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++, np++) {
        q[np].r = o3p[i];
        q[np].s = o3p[j];
        q[np].w = o3w[np];
      }
  }
  for (int g = 0; g < np; g++) {
    const double r = q[g].r, s = q[g].s;
    const double dN[4][2] = {{-0.25 * (1.0 - s), -0.25 * (1.0 - r)},
                             {+0.25 * (1.0 - s), -0.25 * (1.0 + r)},
                             {+0.25 * (1.0 + s), +0.25 * (1.0 + r)},
                             {-0.25 * (1.0 + s), +0.25 * (1.0 - r)}};
    double J[2][2] = {{0}};
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) J[i][j] += dN[a][i] * X[a][j];
    det[g] = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const double s1 = 1.0 / det[g];
    const double Ji[2][2] = {{J[1][1] * s1, -J[0][1] * s1}, {-J[1][0] * s1, J[0][0] * s1}};
    double* G = NiXj + (size_t)g * 8;
    memset(G, 0, sizeof(double) * 8);
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) G[a * 2 + i] += Ji[i][j] * dN[a][j];
    wts[g] = q[g].w;
    if (N) {
      N[g * 4 + 0] = 0.25 * (1.0 - r) * (1.0 - s);
      N[g * 4 + 1] = 0.25 * (1.0 + r) * (1.0 - s);
      N[g * 4 + 2] = 0.25 * (1.0 + r) * (1.0 + s);
      N[g * 4 + 3] = 0.25 * (1.0 - r) * (1.0 + s);
    }
  }
  return np;
}

/* ----------------------------------------------------------------------- */
/* hyperelastic materials (materials_hyperelastic.cpp, solidmech.cpp)       */
/* ----------------------------------------------------------------------- */

enum { M_XX = 0, M_XY, M_XZ, M_YY, M_YZ, M_ZZ };
static const double MAT_I[6] = {1.0, 0.0, 0.0, 1.0, 0.0, 1.0}; /* material.cpp:9 */
static const double MAT_II[6][6] = {{1.0, 0.0, 0.0, 0.0, 0.0, 0.0}, {0.0, 0.5, 0.0, 0.0, 0.0, 0.0},
                                    {0.0, 0.0, 0.5, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 1.0, 0.0, 0.0},
                                    {0.0, 0.0, 0.0, 0.0, 0.5, 0.0}, {0.0, 0.0, 0.0, 0.0, 0.0, 1.0}};

static double J_C(const double* C) {
  return sqrt(C[M_XX] * (C[M_YY] * C[M_ZZ] - C[M_YZ] * C[M_YZ]) -
              C[M_XY] * (C[M_XY] * C[M_ZZ] - C[M_YZ] * C[M_XZ]) +
              C[M_XZ] * (C[M_XY] * C[M_YZ] - C[M_YY] * C[M_XZ]));
}

static void invC_C(const double* C, const double J, double* invC) {
  double oo = 1.0 / (J * J);
  invC[M_XX] = oo * (C[M_YY] * C[M_ZZ] - C[M_YZ] * C[M_YZ]);
  invC[M_XY] = oo * (C[M_XZ] * C[M_YZ] - C[M_XY] * C[M_ZZ]);
  invC[M_XZ] = oo * (C[M_XY] * C[M_YZ] - C[M_XZ] * C[M_YY]);
  invC[M_YY] = oo * (C[M_XX] * C[M_ZZ] - C[M_XZ] * C[M_XZ]);
  invC[M_YZ] = oo * (C[M_XY] * C[M_XZ] - C[M_XX] * C[M_YZ]);
  invC[M_ZZ] = oo * (C[M_XX] * C[M_YY] - C[M_XY] * C[M_XY]);
}

static void IC_C(const double* C, double* IC) {
  IC[0] = C[M_XX] + C[M_YY] + C[M_ZZ];
  IC[1] = C[M_XX] * C[M_YY] + C[M_YY] * C[M_ZZ] + C[M_XX] * C[M_ZZ] - C[M_XY] * C[M_XY] -
          C[M_YZ] * C[M_YZ] - C[M_XZ] * C[M_XZ];
  IC[2] = J_C(C);
}

/* W derivatives: alpha[0..4] = AL_1, AL_2, AL_11, AL_12, AL_22
 * (materials_hyperelastic.cpp:135-204; constants materials_hyperelastic.h:45-105) */
static void W_derivs(int mat_id, const double* MC, double I1, double* alpha) {
  switch (mat_id) {
    case MAT_NH: /* (G, K) */
      alpha[0] = 0.5 * MC[0];
      alpha[1] = 0.0;
      alpha[2] = 0.0;
      alpha[3] = 0.0;
      alpha[4] = 0.0;
      break;
    case MAT_BID: /* (C10, C20, C30, C01, K) */
      alpha[0] = MC[0] + 2 * MC[1] * (I1 - 3.0) + 3 * MC[2] * (I1 - 3.0) * (I1 - 3.0);
      alpha[1] = MC[3];
      alpha[2] = 2 * MC[1] + 6 * MC[2] * (I1 - 3.0);
      alpha[3] = 0.0;
      alpha[4] = 0.0;
      break;
    default: /* Mooney-Rivlin (C10, C01, K) */
      alpha[0] = MC[0];
      alpha[1] = MC[1];
      alpha[2] = 0.0;
      alpha[3] = 0.0;
      alpha[4] = 0.0;
      break;
  }
}

static double mat_K(int mat_id, const double* MC) {
  return mat_id == MAT_NH ? MC[1] : (mat_id == MAT_BID ? MC[4] : MC[2]);
}

/* getS_UP, materials_hyperelastic.cpp:30-62 */
void orc_material_S(int mat_id, const double* MC, const double* C, double press, double* S) {
  double alpha[5];
  double IC[3];
  IC_C(C, IC);
  double _13I1C = 1.0 / 3.0 * IC[0];
  double _23I2C = 2.0 / 3.0 * IC[1];
  double J = IC[2];
  double pp = pow(J, -2.0 / 3.0);
  double pppp = pp * pp;
  double C_inv[6];
  invC_C(C, J, C_inv);
  W_derivs(mat_id, MC, IC[0] * pp, alpha);
  double ko1 = 2 * alpha[0] * pp;
  double ko2 = 2 * alpha[1] * pppp;
  for (int i = 0; i < 6; i++) {
    double A = MAT_I[i] - _13I1C * C_inv[i];
    double B = IC[0] * MAT_I[i] - C[i] - _23I2C * C_inv[i];
    S[i] = ko1 * A + ko2 * B + press * J * C_inv[i];
  }
}

/* getDdDp_UP, materials_hyperelastic.cpp:65-129, for the components comps[0..ncomp):
 * Dd packed upper over (comps[i], comps[j]), j >= i, in that order */
static void material_D_comps(int mat_id, const double* MC, int ncomp, const int* comps,
                             const double* C, double press, double* Dd, double* Dp) {
  double alpha[5];
  double IC[3];
  IC_C(C, IC);
  double _13I1C = 1.0 / 3.0 * IC[0];
  double _23I2C = 2.0 / 3.0 * IC[1];
  double J = IC[2];
  double pp = pow(J, -2.0 / 3.0);
  double oo = pow(J, -2);
  double pppp = pp * pp;
  double C_inv[6];
  invC_C(C, J, C_inv);
  W_derivs(mat_id, MC, IC[0] * pp, alpha);
  double A[6], B[6];
  for (int i = 0; i < 6; i++) {
    A[i] = MAT_I[i] - _13I1C * C_inv[i];
    B[i] = IC[0] * MAT_I[i] - C[i] - _23I2C * C_inv[i];
  }
  const double* c = C_inv;
  double IIt[6][6] = {
      {-c[M_XX] * c[M_XX], -c[M_XX] * c[M_XY], -c[M_XX] * c[M_XZ], -c[M_XY] * c[M_XY],
       -c[M_XY] * c[M_XZ], -c[M_XZ] * c[M_XZ]},
      {-c[M_XX] * c[M_XY], -0.5 * (c[M_XX] * c[M_YY] + c[M_XY] * c[M_XY]),
       -0.5 * (c[M_XX] * c[M_YZ] + c[M_XZ] * c[M_XY]), -c[M_XY] * c[M_YY],
       -0.5 * (c[M_XY] * c[M_YZ] + c[M_XZ] * c[M_YY]), -c[M_XZ] * c[M_YZ]},
      {-c[M_XX] * c[M_XZ], -0.5 * (c[M_XX] * c[M_YZ] + c[M_XY] * c[M_XZ]),
       -0.5 * (c[M_XX] * c[M_ZZ] + c[M_XZ] * c[M_XZ]), -c[M_XY] * c[M_YZ],
       -0.5 * (c[M_XY] * c[M_ZZ] + c[M_XZ] * c[M_YZ]), -c[M_XZ] * c[M_ZZ]},
      {-c[M_XY] * c[M_XY], -c[M_XY] * c[M_YY], -c[M_XY] * c[M_YZ], -c[M_YY] * c[M_YY],
       -c[M_YY] * c[M_YZ], -c[M_YZ] * c[M_YZ]},
      {-c[M_XY] * c[M_XZ], -0.5 * (c[M_XY] * c[M_YZ] + c[M_YY] * c[M_XZ]),
       -0.5 * (c[M_XY] * c[M_ZZ] + c[M_YZ] * c[M_XZ]), -c[M_YY] * c[M_YZ],
       -0.5 * (c[M_YY] * c[M_ZZ] + c[M_YZ] * c[M_YZ]), -c[M_YZ] * c[M_ZZ]},
      {-c[M_XZ] * c[M_XZ], -c[M_XZ] * c[M_YZ], -c[M_XZ] * c[M_ZZ], -c[M_YZ] * c[M_YZ],
       -c[M_YZ] * c[M_ZZ], -c[M_ZZ] * c[M_ZZ]}};
  int ind = 0;
  for (int i = 0; i < ncomp; i++) {
    const int ij = comps[i];
    for (int j = i; j < ncomp; j++) {
      const int kl = comps[j];
      Dd[ind] = 4.0 * alpha[2] * pppp * A[ij] * A[kl] +
                4.0 * alpha[3] * oo * (B[ij] * A[kl] + A[ij] * B[kl]) +
                4.0 * alpha[4] * pppp * pppp * B[ij] * B[kl] -
                4.0 / 3.0 * alpha[0] * pp *
                    (C_inv[ij] * A[kl] + A[ij] * C_inv[kl] + _13I1C * C_inv[ij] * C_inv[kl] +
                     IC[0] * IIt[ij][kl]) -
                8.0 / 3.0 * alpha[1] * pppp *
                    (C_inv[ij] * B[kl] + B[ij] * C_inv[kl] + _23I2C * C_inv[ij] * C_inv[kl] -
                     3.0 / 2.0 * MAT_I[ij] * MAT_I[kl] + 3.0 / 2.0 * MAT_II[ij][kl] +
                     IC[1] * IIt[ij][kl]) +
                press * J * (C_inv[ij] * C_inv[kl] + 2 * IIt[ij][kl]);
      Dd[ind] = Dd[ind] / 2.0;
      ind++;
    }
    Dp[i] = J * C_inv[ij];
  }
}

void orc_material_D(int mat_id, const double* MC, const double* C, double press, double* Dd,
                    double* Dp) {
  static const int all[6] = {0, 1, 2, 3, 4, 5};
  material_D_comps(mat_id, MC, 6, all, C, press, Dd, Dp);
}

/* ----------------------------------------------------------------------- */
/* model                                                                    */
/* ----------------------------------------------------------------------- */

typedef struct {
  uint32_t rows, cols, nnz, max_in_row;
  uint32_t* iofeir;
  uint32_t* columns;
  double* values;
  int compressed;
} csr_block;

typedef struct {
  uint32_t node;
  int dof;
  double coef;
} mpc_term;

typedef struct {
  mpc_term t[5];
  double b;
  uint32_t eq;
} mpc_eq;

typedef struct {
  uint32_t master;
  uint32_t n_slaves, n_dofs;
  uint32_t* slaves;
  int dofs[3];
  uint32_t first_mpc; /* index into model mpcs */
} rigid_body;

struct orc_model {
  int etype, mat_id, npe;
  double MC[5];
  uint32_t n_nodes, n_elems;
  double* xyz;
  uint32_t* conn;
  double* eparams;
  /* DoF tables */
  uint8_t* node_mask;
  uint8_t* elem_mask;
  uint8_t* node_fix;
  uint32_t* node_eq;
  uint32_t* elem_eq;
  uint32_t n_dofs, n_con, n_unk, n_mpc;
  /* constraints / MPC */
  uint32_t n_fix;
  uint32_t* fix_node;
  int* fix_dof;
  rigid_body* rbs;
  uint32_t n_rbs;
  mpc_eq* mpcs;     /* rigid-body MPC equations (n_rmpc) */
  uint32_t n_rmpc;
  /* linear MPC equations added with orc_add_mpc (FEStorage::addMpc), numbered
   * before the rigid-body ones: terms lm_ptr[k] .. lm_ptr[k+1] */
  uint32_t n_lmpc, lm_terms;
  uint32_t* lm_ptr;
  uint32_t* lm_node;
  int* lm_dof;
  double* lm_coef;
  double* lm_b;
  uint32_t* lm_eq;
  /* SurfaceLINETH elements (QUADTH.h:38-55), numbered after the n_elems
   * elements: line_conn 2 per line, line_par (htc, flux, etemp0, etemp1) */
  uint32_t n_lines;
  uint32_t* line_conn;
  double* line_par;
  /* FEStorage::setTransient: C and M on K's pattern (FEStorage.cpp:475-480) */
  int transient;
  double* cval[3];
  double* mval[3];
  /* global system */
  csr_block blk[3]; /* block(1), block(1,2), block(2) */
  double* U;
  double* F;
  /* element state */
  int np;
  double* NiXj; /* E x np x npe x dim */
  double* det;  /* E x np */
  double* wts;  /* np */
  double* Nq;   /* np x npe (QUADTH) */
  double* S;    /* E x np x 6 */
  double* Cst;  /* E x np x 6 */
  double* O;    /* E x np x 9 */
  int setup_done;
  char err[256];
};

static int fail(orc_model* m, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(m->err, sizeof(m->err), fmt, ap);
  va_end(ap);
  return 1;
}

orc_model* orc_new(int elem_type, uint32_t n_nodes, const double* xyz, uint32_t n_elems,
                   const uint32_t* conn, int mat_id, const double* mat_c, int n_mat_c,
                   const double* elem_params, int n_elem_params) {
  orc_model* m = (orc_model*)calloc(1, sizeof(orc_model));
  m->etype = elem_type;
  m->npe = elem_type == ET_SOLID81 ? 8 : 4;
  m->mat_id = mat_id;
  for (int i = 0; i < n_mat_c && i < 5; i++) m->MC[i] = mat_c[i];
  m->n_nodes = n_nodes;
  m->n_elems = n_elems;
  m->xyz = (double*)malloc(sizeof(double) * 3 * (n_nodes ? n_nodes : 1));
  memcpy(m->xyz, xyz, sizeof(double) * 3 * n_nodes);
  m->conn = (uint32_t*)malloc(sizeof(uint32_t) * m->npe * (n_elems ? n_elems : 1));
  memcpy(m->conn, conn, sizeof(uint32_t) * m->npe * n_elems);
  m->eparams = (double*)calloc((size_t)EPAR * (n_elems ? n_elems : 1), sizeof(double));
  if (elem_params && n_elem_params > 0)
    for (uint32_t e = 0; e < n_elems; e++)
      for (int k = 0; k < n_elem_params && k < EPAR; k++)
        m->eparams[(size_t)e * EPAR + k] = elem_params[(size_t)e * n_elem_params + k];
  return m;
}

void orc_free(orc_model* m) {
  if (!m) return;
  free(m->xyz); free(m->conn); free(m->eparams);
  free(m->line_conn); free(m->line_par);
  for (int b = 0; b < 3; b++) {
    free(m->cval[b]); free(m->mval[b]);
  }
  free(m->node_mask); free(m->elem_mask); free(m->node_fix); free(m->node_eq); free(m->elem_eq);
  free(m->fix_node); free(m->fix_dof);
  for (uint32_t i = 0; i < m->n_rbs; i++) free(m->rbs[i].slaves);
  free(m->rbs); free(m->mpcs);
  free(m->lm_ptr); free(m->lm_node); free(m->lm_dof); free(m->lm_coef); free(m->lm_b);
  free(m->lm_eq);
  for (int b = 0; b < 3; b++) {
    free(m->blk[b].iofeir); free(m->blk[b].columns); free(m->blk[b].values);
  }
  free(m->U); free(m->F); free(m->NiXj); free(m->det); free(m->wts); free(m->Nq);
  free(m->S); free(m->Cst); free(m->O);
  free(m);
}

const char* orc_error(orc_model* m) { return m->err; }

int orc_add_fix(orc_model* m, uint32_t n, const uint32_t* nodes, const int32_t* dofs) {
  m->fix_node = (uint32_t*)realloc(m->fix_node, sizeof(uint32_t) * (m->n_fix + n));
  m->fix_dof = (int*)realloc(m->fix_dof, sizeof(int) * (m->n_fix + n));
  for (uint32_t i = 0; i < n; i++) {
    m->fix_node[m->n_fix + i] = nodes[i];
    m->fix_dof[m->n_fix + i] = dofs[i];
  }
  m->n_fix += n;
  return 0;
}

int orc_add_rigid_body(orc_model* m, uint32_t master, uint32_t n_slaves, const uint32_t* slaves,
                       uint32_t n_dofs, const int32_t* dofs) {
  if (n_dofs > 3) return fail(m, "rigid body: at most 3 slave DoFs");
  m->rbs = (rigid_body*)realloc(m->rbs, sizeof(rigid_body) * (m->n_rbs + 1));
  rigid_body* rb = &m->rbs[m->n_rbs++];
  rb->master = master;
  rb->n_slaves = n_slaves;
  rb->n_dofs = n_dofs;
  rb->slaves = (uint32_t*)malloc(sizeof(uint32_t) * (n_slaves ? n_slaves : 1));
  memcpy(rb->slaves, slaves, sizeof(uint32_t) * n_slaves);
  for (uint32_t i = 0; i < n_dofs; i++) rb->dofs[i] = dofs[i];
  return 0;
}

/* FEStorage::addMpc (FEStorage.cpp:175-179) of an Mpc with these terms */
int orc_add_mpc(orc_model* m, uint32_t n_terms, const uint32_t* nodes, const int32_t* dofs,
                const double* coefs, double b) {
  if (!n_terms) return fail(m, "MPC without terms");
  const uint32_t k = m->n_lmpc, t0 = m->lm_terms;
  m->lm_ptr = (uint32_t*)realloc(m->lm_ptr, sizeof(uint32_t) * (k + 2));
  m->lm_b = (double*)realloc(m->lm_b, sizeof(double) * (k + 1));
  m->lm_eq = (uint32_t*)realloc(m->lm_eq, sizeof(uint32_t) * (k + 1));
  m->lm_node = (uint32_t*)realloc(m->lm_node, sizeof(uint32_t) * (t0 + n_terms));
  m->lm_dof = (int*)realloc(m->lm_dof, sizeof(int) * (t0 + n_terms));
  m->lm_coef = (double*)realloc(m->lm_coef, sizeof(double) * (t0 + n_terms));
  if (k == 0) m->lm_ptr[0] = 0;
  for (uint32_t t = 0; t < n_terms; t++) {
    m->lm_node[t0 + t] = nodes[t];
    m->lm_dof[t0 + t] = dofs[t];
    m->lm_coef[t0 + t] = coefs[t];
  }
  m->lm_terms = t0 + n_terms;
  m->lm_ptr[k + 1] = m->lm_terms;
  m->lm_b[k] = b;
  m->lm_eq[k] = 0;
  m->n_lmpc = k + 1;
  return 0;
}

/* SparsityInfo::reinit / addEntry / compress (SparseMatrix.cpp:44-114) */
static void blk_init(csr_block* b, uint32_t rows, uint32_t cols, uint32_t max_in_row) {
  b->rows = rows;
  b->cols = cols;
  b->max_in_row = max_in_row < cols ? max_in_row : cols;
  const size_t cap = (size_t)rows * b->max_in_row;
  b->columns = (uint32_t*)malloc(sizeof(uint32_t) * (cap ? cap : 1));
  for (size_t i = 0; i < cap; i++) b->columns[i] = INVALID;
  b->iofeir = (uint32_t*)malloc(sizeof(uint32_t) * (rows + 1));
  b->iofeir[0] = 1;
  for (uint32_t i = 1; i <= rows; i++) b->iofeir[i] = b->iofeir[i - 1] + b->max_in_row;
  b->nnz = 0;
  b->compressed = 0;
}

static int blk_add_entry(orc_model* m, csr_block* b, uint32_t i, uint32_t j) {
  uint32_t st = b->iofeir[i - 1] - 1, en = b->iofeir[i] - 1;
  for (uint32_t k = st; k < en; k++) {
    if (b->columns[k] == j) return 0;
    if (b->columns[k] == INVALID) {
      b->columns[k] = j;
      b->nnz++;
      return 0;
    }
  }
  return fail(m, "maxInRow overflow!");
}

static int cmp_u32(const void* a, const void* b) {
  uint32_t x = *(const uint32_t*)a, y = *(const uint32_t*)b;
  return x < y ? -1 : (x > y ? 1 : 0);
}

static void blk_compress(csr_block* b) {
  uint32_t next = 0, next_row = 0;
  uint32_t* old = b->columns;
  b->columns = (uint32_t*)malloc(sizeof(uint32_t) * (b->nnz ? b->nnz : 1));
  for (uint32_t i = 0; i < b->rows; i++) {
    for (uint32_t j = b->iofeir[i] - 1; j < b->iofeir[i + 1] - 1; j++) {
      if (old[j] == INVALID) break;
      b->columns[next++] = old[j];
    }
    if (next - next_row > 1) qsort(&b->columns[next_row], next - next_row, sizeof(uint32_t), cmp_u32);
    b->iofeir[i] = next_row + 1;
    next_row = next;
  }
  b->iofeir[b->rows] = next + 1;
  free(old);
  b->values = (double*)calloc(b->nnz ? b->nnz : 1, sizeof(double));
  b->compressed = 1;
}

/* SparsityInfo::getIndex (SparseMatrix.cpp:117-154) */
static uint32_t blk_index(const csr_block* b, uint32_t i, uint32_t j) {
  uint32_t ind;
  uint32_t st = b->iofeir[i - 1] - 1;
  uint32_t en = b->iofeir[i] - 1;
  if (st == en) return INVALID;
  en--;
  for (;;) {
    if (en - st == 1) {
      if (b->columns[st] == j) return st;
      if (b->columns[en] == j) return en;
      return INVALID;
    }
    ind = (uint32_t)((en + st) * 0.5);
    if (b->columns[ind] == j) return ind;
    if (en == st) return INVALID;
    if (b->columns[ind] > j)
      en = ind;
    else
      st = ind;
  }
}

/* BlockSparseSymMatrix<2>::getBlockAndPosition + routing (BlockSparseMatrix.h:126-168);
 * returns the block slot 0 (block 1), 1 (block 1,2), 2 (block 2). */
static int route(const orc_model* m, uint32_t* i, uint32_t* j) {
  if (*i > *j) {
    uint32_t t = *i;
    *i = *j;
    *j = t;
  }
  const uint32_t nc = m->n_con;
  int bi = *i <= nc ? 1 : 2, bj = *j <= nc ? 1 : 2;
  if (bi == 2) *i -= nc;
  if (bj == 2) *j -= nc;
  if (bi == bj) return bi == 1 ? 0 : 2;
  return 1;
}

static int add_entry(orc_model* m, uint32_t i, uint32_t j) {
  int b = route(m, &i, &j);
  return blk_add_entry(m, &m->blk[b], i, j);
}

/* value arrays: NULL = K's own; C and M share K's pattern (FEStorage.cpp:475-480) */
static int add_value_to(orc_model* m, double** vals, uint32_t i, uint32_t j, double v) {
  int b = route(m, &i, &j);
  uint32_t idx = blk_index(&m->blk[b], i, j);
  if (idx == INVALID) return fail(m, "The position(%u, %u) is absent in the matrix", i, j);
  (vals ? vals[b] : m->blk[b].values)[idx] += v;
  return 0;
}

static int add_value(orc_model* m, uint32_t i, uint32_t j, double v) {
  return add_value_to(m, NULL, i, j, v);
}

/* nodes of element en (1-based): the n_elems elements, then the lines */
static inline int elem_npe(const orc_model* m, uint32_t en) {
  return en <= m->n_elems ? m->npe : 2;
}
static inline uint32_t elem_node(const orc_model* m, uint32_t en, int a) {
  if (en <= m->n_elems) return m->conn[(size_t)(en - 1) * m->npe + a];
  return m->line_conn[2 * (size_t)(en - 1 - m->n_elems) + a];
}

static inline uint32_t neq(const orc_model* m, uint32_t node, int dof) {
  return m->node_eq[(size_t)(node - 1) * NDOFT + dof];
}
static inline uint32_t eeq(const orc_model* m, uint32_t el, int dof) {
  return m->elem_eq[(size_t)(el - 1) * NDOFT + dof];
}

int orc_setup(orc_model* m, uint32_t max_in_row) {
  const uint32_t N = m->n_nodes, E = m->n_elems, L = m->n_lines, EL = E + L;
  if (N < 1 && E < 1) return fail(m, "No any nodes or elements");
  if (m->transient && m->etype != ET_QUADTH)
    return fail(m, "transient: only QUADTH builds C and M here");
  m->node_mask = (uint8_t*)calloc(N + 1, 1);
  m->elem_mask = (uint8_t*)calloc(EL + 1, 1);
  m->node_fix = (uint8_t*)calloc(N + 1, 1);
  m->node_eq = (uint32_t*)calloc((size_t)(N + 1) * NDOFT, sizeof(uint32_t));
  m->elem_eq = (uint32_t*)calloc((size_t)(EL + 1) * NDOFT, sizeof(uint32_t));

  /* --- Element::pre(): DoF registration and element state (SOLID81.cpp:12-26,
   *     TETRA0.cpp:10-14, QUADTH.cpp:12-20) --- */
  for (uint32_t e = 0; e < E; e++) {
    const uint32_t* c = m->conn + (size_t)e * m->npe;
    for (int a = 0; a < m->npe; a++) {
      if (c[a] < 1 || c[a] > N) return fail(m, "element %u: bad node id", e + 1);
      if (m->etype == ET_QUADTH)
        m->node_mask[c[a] - 1] |= 1u << TEMP;
      else if (m->etype == ET_PLANE41)  /* PLANE41.cpp:25-27 */
        m->node_mask[c[a] - 1] |= (1u << UX) | (1u << UY);
      else
        m->node_mask[c[a] - 1] |= (1u << UX) | (1u << UY) | (1u << UZ);
    }
    if (m->etype == ET_SOLID81 || m->etype == ET_PLANE41)
      m->elem_mask[e] |= 1u << HYDRO_PRESSURE;
  }
  /* SurfaceLINETH::pre (QUADTH.cpp:73-84): TEMP on both nodes; a zero second
   * environment temperature takes the first */
  for (uint32_t l = 0; l < L; l++) {
    for (int a = 0; a < 2; a++) {
      const uint32_t n = m->line_conn[2 * l + a];
      if (n < 1 || n > N) return fail(m, "line %u: bad node id", l + 1);
      m->node_mask[n - 1] |= 1u << TEMP;
    }
    if (m->line_par[4 * l + 3] == 0.0) m->line_par[4 * l + 3] = m->line_par[4 * l + 2];
  }
  if (m->etype == ET_SOLID81) {
    m->np = 8;
    m->NiXj = (double*)malloc(sizeof(double) * (size_t)E * 8 * 24 + 8);
    m->det = (double*)malloc(sizeof(double) * (size_t)E * 8 + 8);
    m->wts = (double*)malloc(sizeof(double) * 8);
    m->S = (double*)calloc((size_t)E * 8 * 6 + 1, sizeof(double));
    m->Cst = (double*)calloc((size_t)E * 8 * 6 + 1, sizeof(double));
    m->O = (double*)calloc((size_t)E * 8 * 9 + 1, sizeof(double));
    for (uint32_t e = 0; e < E; e++) {
      double X[8][3];
      for (int a = 0; a < 8; a++)
        for (int d = 0; d < 3; d++) X[a][d] = m->xyz[(size_t)(m->conn[e * 8 + a] - 1) * 3 + d];
      hex_jacobian(X, 2, m->NiXj + (size_t)e * 8 * 24, m->det + (size_t)e * 8, m->wts);
      for (int g = 0; g < 8; g++) {
        double* C = m->Cst + ((size_t)e * 8 + g) * 6;
        C[0] = 1.0; C[3] = 1.0; C[5] = 1.0;
      }
    }
  } else if (m->etype == ET_QUADTH || m->etype == ET_PLANE41) {
    m->np = 4;
    if (m->etype == ET_PLANE41) {
      /* PLANE41::pre (PLANE41.cpp:15-24): S = 0, C = (1, 1, 0), O = 0 */
      m->S = (double*)calloc((size_t)E * 4 * 3 + 1, sizeof(double));
      m->Cst = (double*)calloc((size_t)E * 4 * 3 + 1, sizeof(double));
      m->O = (double*)calloc((size_t)E * 4 * 4 + 1, sizeof(double));
      for (size_t g = 0; g < (size_t)E * 4; g++) {
        m->Cst[g * 3 + 0] = 1.0;
        m->Cst[g * 3 + 1] = 1.0;
      }
    }
    m->NiXj = (double*)malloc(sizeof(double) * (size_t)E * 4 * 8 + 8);
    m->det = (double*)malloc(sizeof(double) * (size_t)E * 4 + 8);
    m->wts = (double*)malloc(sizeof(double) * 4);
    m->Nq = (double*)malloc(sizeof(double) * 16);
    for (uint32_t e = 0; e < E; e++) {
      double X[4][3];
      for (int a = 0; a < 4; a++)
        for (int d = 0; d < 3; d++) X[a][d] = m->xyz[(size_t)(m->conn[e * 4 + a] - 1) * 3 + d];
      quad_jacobian(X, 2, m->NiXj + (size_t)e * 32, m->det + (size_t)e * 4, m->wts, m->Nq);
    }
  }

  /* --- RigidBodyMpc::pre + registerMpcsInStorage (Mpc.cpp:30-68) --- */
  uint32_t total_mpc = 0;
  for (uint32_t r = 0; r < m->n_rbs; r++) total_mpc += m->rbs[r].n_slaves * m->rbs[r].n_dofs;
  m->mpcs = (mpc_eq*)calloc(total_mpc + 1, sizeof(mpc_eq));
  m->n_rmpc = total_mpc;
  m->n_mpc = m->n_lmpc + total_mpc;
  {
    uint32_t k = 0;
    for (uint32_t r = 0; r < m->n_rbs; r++) {
      rigid_body* rb = &m->rbs[r];
      rb->first_mpc = k;
      for (uint32_t s = 0; s < rb->n_slaves; s++)
        for (uint32_t d = 0; d < rb->n_dofs; d++, k++) {
          mpc_eq* q = &m->mpcs[k];
          q->b = 0.0;
          q->t[0] = (mpc_term){rb->slaves[s], rb->dofs[d], 1.0};
          q->t[1] = (mpc_term){rb->master, rb->dofs[d], -1.0};
          q->t[2] = (mpc_term){rb->master, ROTX, 0.0};
          q->t[3] = (mpc_term){rb->master, ROTY, 0.0};
          q->t[4] = (mpc_term){rb->master, ROTZ, 0.0};
        }
      m->node_mask[rb->master - 1] |= 0x3F; /* UX..ROTZ */
    }
  }

  m->n_dofs = 0;
  for (uint32_t n = 0; n < N; n++) m->n_dofs += (uint32_t)__builtin_popcount(m->node_mask[n]);
  for (uint32_t e = 0; e < E; e++) m->n_dofs += (uint32_t)__builtin_popcount(m->elem_mask[e]);
  if (!m->n_dofs) return fail(m, "CHECK failed: _nDofs");

  /* --- setConstrainedNodeDof (FEStorage.cpp:81-90) --- */
  m->n_con = 0;
  for (uint32_t f = 0; f < m->n_fix; f++) {
    uint32_t n = m->fix_node[f];
    int d = m->fix_dof[f];
    if (n < 1 || n > N || !(m->node_mask[n - 1] & (1u << d))) return fail(m, "fix of unused DoF");
    if (!(m->node_fix[n - 1] & (1u << d))) {
      m->node_fix[n - 1] |= (uint8_t)(1u << d);
      m->n_con++;
    }
  }

  /* --- assignEquationNumbers (FEStorage.cpp:382-432) --- */
  m->n_unk = m->n_dofs - m->n_con;
  if (!m->n_unk) return fail(m, "CHECK failed: _nUnknownDofs");
  uint32_t next_solve = m->n_con + 1, next_const = 1;
  for (uint32_t e = 0; e < E; e++)
    for (int t = 0; t < NDOFT; t++)
      if (m->elem_mask[e] & (1u << t)) m->elem_eq[(size_t)e * NDOFT + t] = next_solve++;
  for (uint32_t n = 0; n < N; n++)
    for (int t = 0; t < NDOFT; t++)
      if (m->node_mask[n] & (1u << t))
        m->node_eq[(size_t)n * NDOFT + t] =
            (m->node_fix[n] & (1u << t)) ? next_const++ : next_solve++;
  /* mpcs list order: addMpc'd equations, then the collections' (initDofs) */
  for (uint32_t k = 0; k < m->n_lmpc; k++) {
    for (uint32_t t = m->lm_ptr[k]; t < m->lm_ptr[k + 1]; t++) {
      const uint32_t n = m->lm_node[t];
      const int d = m->lm_dof[t];
      if (n < 1 || n > N || d < 0 || d >= NDOFT || !(m->node_mask[n - 1] & (1u << d)))
        return fail(m, "MPC term on an unused DoF");
    }
    m->lm_eq[k] = next_solve++;
  }
  for (uint32_t k = 0; k < m->n_rmpc; k++) m->mpcs[k].eq = next_solve++;

  /* --- initSolutionData (FEStorage.cpp:434-550) --- */
  const uint32_t nc = m->n_con, ns = m->n_unk + m->n_mpc;
  blk_init(&m->blk[0], nc, nc, max_in_row);
  blk_init(&m->blk[1], nc, ns, max_in_row);
  blk_init(&m->blk[2], ns, ns, max_in_row);
  const uint32_t ntot = m->n_dofs + m->n_mpc;
  m->U = (double*)calloc(ntot + 1, sizeof(double));
  m->F = (double*)calloc(ntot + 1, sizeof(double));

  /* learnTopology: node -> ascending element ids (FEStorage.cpp:580-589);
   * the lines are elements E+1 .. E+L */
  uint32_t* cnt = (uint32_t*)calloc(N + 1, sizeof(uint32_t));
  for (uint32_t e = 0; e < EL; e++)
    for (int a = 0; a < elem_npe(m, e + 1); a++) cnt[elem_node(m, e + 1, a)]++;
  for (uint32_t n = 1; n <= N; n++) cnt[n] += cnt[n - 1];
  uint32_t* topo = (uint32_t*)malloc(sizeof(uint32_t) * (cnt[N] + 1));
  uint32_t* fillp = (uint32_t*)malloc(sizeof(uint32_t) * (N + 1));
  memcpy(fillp, cnt, sizeof(uint32_t) * (N + 1));
  for (uint32_t e = 0; e < EL; e++)
    for (int a = 0; a < elem_npe(m, e + 1); a++) {
      uint32_t n = elem_node(m, e + 1, a);
      uint32_t* beg = topo + cnt[n - 1];
      int dup = 0;
      for (uint32_t* p = beg; p < topo + fillp[n - 1]; p++) dup |= (*p == e + 1);
      if (!dup) topo[fillp[n - 1]++] = e + 1;
    }
  int rc = 0;
  for (uint32_t nn = 1; nn <= N && !rc; nn++) {
    const uint8_t mn = m->node_mask[nn - 1];
    for (uint32_t* pe = topo + cnt[nn - 1]; pe < topo + fillp[nn - 1] && !rc; pe++) {
      const uint32_t en = *pe;
      const uint8_t me = m->elem_mask[en - 1];
      for (int t1 = 0; t1 < NDOFT; t1++)
        if (me & (1u << t1))
          for (int t2 = 0; t2 < NDOFT; t2++)
            if (mn & (1u << t2)) rc |= add_entry(m, eeq(m, en, t1), neq(m, nn, t2));
      for (int a = 0; a < elem_npe(m, en); a++) {
        uint32_t nn2 = elem_node(m, en, a);
        if (nn2 < nn) continue;
        const uint8_t m2 = m->node_mask[nn2 - 1];
        for (int t1 = 0; t1 < NDOFT; t1++)
          if (m2 & (1u << t1))
            for (int t2 = 0; t2 < NDOFT; t2++)
              if (mn & (1u << t2)) rc |= add_entry(m, neq(m, nn2, t1), neq(m, nn, t2));
      }
    }
  }
  free(cnt); free(topo); free(fillp);
  for (uint32_t en = 1; en <= E && !rc; en++) {
    const uint8_t me = m->elem_mask[en - 1];
    for (int t1 = 0; t1 < NDOFT; t1++)
      if (me & (1u << t1))
        for (int t2 = 0; t2 < NDOFT; t2++)
          if (me & (1u << t2)) rc |= add_entry(m, eeq(m, en, t1), eeq(m, en, t2));
  }
  for (uint32_t k = 0; k < m->n_lmpc && !rc; k++)
    for (uint32_t t = m->lm_ptr[k]; t < m->lm_ptr[k + 1]; t++)
      rc |= add_entry(m, m->lm_eq[k], neq(m, m->lm_node[t], m->lm_dof[t]));
  for (uint32_t k = 0; k < m->n_rmpc && !rc; k++)
    for (int t = 0; t < 5; t++) {
      uint32_t eqj = neq(m, m->mpcs[k].t[t].node, m->mpcs[k].t[t].dof);
      rc |= add_entry(m, m->mpcs[k].eq, eqj);
    }
  if (rc) return 1;
  for (int b = 0; b < 3; b++) blk_compress(&m->blk[b]);
  if (m->transient)
    for (int b = 0; b < 3; b++) {
      m->cval[b] = (double*)calloc(m->blk[b].nnz ? m->blk[b].nnz : 1, sizeof(double));
      m->mval[b] = (double*)calloc(m->blk[b].nnz ? m->blk[b].nnz : 1, sizeof(double));
    }
  m->setup_done = 1;
  return 0;
}

void orc_info(orc_model* m, uint32_t* out) {
  out[0] = m->n_dofs;
  out[1] = m->n_con;
  out[2] = m->n_unk;
  out[3] = m->n_mpc;
  for (int b = 0; b < 3; b++) {
    out[4 + 3 * b] = m->blk[b].rows;
    out[5 + 3 * b] = m->blk[b].cols;
    out[6 + 3 * b] = m->blk[b].nnz;
  }
}

static int slot_of(int block) { return block == 1 ? 0 : (block == 2 ? 2 : 1); }

int orc_pattern(orc_model* m, int block, uint32_t* iofeir, uint32_t* columns) {
  csr_block* b = &m->blk[slot_of(block)];
  if (b->rows == 0 && b->nnz == 0) return 0;
  memcpy(iofeir, b->iofeir, sizeof(uint32_t) * (b->rows + 1));
  memcpy(columns, b->columns, sizeof(uint32_t) * b->nnz);
  return 0;
}

int orc_eq_numbers(orc_model* m, uint32_t* node_eq, uint32_t* elem_eq) {
  memcpy(node_eq, m->node_eq, sizeof(uint32_t) * (size_t)m->n_nodes * NDOFT);
  memcpy(elem_eq, m->elem_eq, sizeof(uint32_t) * (size_t)m->n_elems * NDOFT);
  return 0;
}

int orc_set_U(orc_model* m, const double* U, uint32_t n) {
  if (n != m->n_dofs + m->n_mpc) return fail(m, "U size mismatch");
  memcpy(m->U, U, sizeof(double) * n);
  return 0;
}

/* ----------------------------------------------------------------------- */
/* SOLID81 (SOLID81.cpp)                                                    */
/* ----------------------------------------------------------------------- */

static void make_B_NL(const double* G /*8x3*/, double* B /*9x24*/) {
  for (int i = 0; i < 8; i++) {
    B[0 * 24 + (i * 3 + 0)] += G[i * 3 + 0];
    B[1 * 24 + (i * 3 + 0)] += G[i * 3 + 1];
    B[2 * 24 + (i * 3 + 0)] += G[i * 3 + 2];
    B[3 * 24 + (i * 3 + 1)] += G[i * 3 + 0];
    B[4 * 24 + (i * 3 + 1)] += G[i * 3 + 1];
    B[5 * 24 + (i * 3 + 1)] += G[i * 3 + 2];
    B[6 * 24 + (i * 3 + 2)] += G[i * 3 + 0];
    B[7 * 24 + (i * 3 + 2)] += G[i * 3 + 1];
    B[8 * 24 + (i * 3 + 2)] += G[i * 3 + 2];
  }
}

static void make_B_L(const double* G, double* B /*6x24*/) {
  for (int i = 0; i < 8; i++) {
    B[0 * 24 + (i * 3 + 0)] += 2 * G[i * 3 + 0];
    B[1 * 24 + (i * 3 + 0)] += 2 * G[i * 3 + 1];
    B[1 * 24 + (i * 3 + 1)] += 2 * G[i * 3 + 0];
    B[2 * 24 + (i * 3 + 0)] += 2 * G[i * 3 + 2];
    B[2 * 24 + (i * 3 + 2)] += 2 * G[i * 3 + 0];
    B[3 * 24 + (i * 3 + 1)] += 2 * G[i * 3 + 1];
    B[4 * 24 + (i * 3 + 1)] += 2 * G[i * 3 + 2];
    B[4 * 24 + (i * 3 + 2)] += 2 * G[i * 3 + 1];
    B[5 * 24 + (i * 3 + 2)] += 2 * G[i * 3 + 2];
  }
}

static void make_S9(const double* S, double* Sp /*packed 9x9: 45*/) {
  Sp[0] += S[M_XX]; Sp[1] += S[M_XY]; Sp[2] += S[M_XZ];
  Sp[9] += S[M_YY]; Sp[10] += S[M_YZ]; Sp[17] += S[M_ZZ];
  Sp[24] += S[M_XX]; Sp[25] += S[M_XY]; Sp[26] += S[M_XZ];
  Sp[30] += S[M_YY]; Sp[31] += S[M_YZ]; Sp[35] += S[M_ZZ];
  Sp[39] += S[M_XX]; Sp[40] += S[M_XY]; Sp[41] += S[M_XZ];
  Sp[42] += S[M_YY]; Sp[43] += S[M_YZ]; Sp[44] += S[M_ZZ];
}

static void make_Omega(const double* O, double* W /*6x9*/) {
  for (int i = 0; i < 3; i++) {
    W[0 * 9 + (i * 3 + 0)] = O[0 + i * 3];
    W[1 * 9 + (i * 3 + 0)] = O[1 + i * 3];
    W[1 * 9 + (i * 3 + 1)] = O[0 + i * 3];
    W[2 * 9 + (i * 3 + 0)] = O[2 + i * 3];
    W[2 * 9 + (i * 3 + 2)] = O[0 + i * 3];
    W[3 * 9 + (i * 3 + 1)] = O[1 + i * 3];
    W[4 * 9 + (i * 3 + 1)] = O[2 + i * 3];
    W[4 * 9 + (i * 3 + 2)] = O[1 + i * 3];
    W[5 * 9 + (i * 3 + 2)] = O[2 + i * 3];
  }
}

static void solid81_update(orc_model* m, uint32_t e) {
  double U[24];
  const uint32_t* c = m->conn + (size_t)e * 8;
  for (int i = 0; i < 8; i++)
    for (int d = 0; d < 3; d++) U[i * 3 + d] = m->U[neq(m, c[i], d) - 1];
  const double p_e = m->U[eeq(m, e + 1, HYDRO_PRESSURE) - 1];
  for (int g = 0; g < 8; g++) {
    double B_NL[9 * 24];
    memset(B_NL, 0, sizeof(B_NL));
    make_B_NL(m->NiXj + ((size_t)e * 8 + g) * 24, B_NL);
    double* O = m->O + ((size_t)e * 8 + g) * 9;
    memset(O, 0, sizeof(double) * 9);
    k_matBVprod(9, 24, B_NL, U, 1.0, O);
    double* C = m->Cst + ((size_t)e * 8 + g) * 6;
    C[M_XX] = 1.0 + 2 * O[0] + pow(O[0], 2) + pow(O[3], 2) + pow(O[6], 2);
    C[M_YY] = 1.0 + 2 * O[4] + pow(O[1], 2) + pow(O[4], 2) + pow(O[7], 2);
    C[M_ZZ] = 1.0 + 2 * O[8] + pow(O[2], 2) + pow(O[5], 2) + pow(O[8], 2);
    C[M_XY] = O[1] + O[3] + O[0] * O[1] + O[3] * O[4] + O[6] * O[7];
    C[M_YZ] = O[5] + O[7] + O[1] * O[2] + O[4] * O[5] + O[7] * O[8];
    C[M_XZ] = O[2] + O[6] + O[0] * O[2] + O[3] * O[5] + O[6] * O[8];
    orc_material_S(m->mat_id, m->MC, C, p_e, m->S + ((size_t)e * 8 + g) * 6);
  }
}

static int solid81_buildK(orc_model* m, uint32_t e) {
  double Kpp = 0.0, Fp = 0.0;
  double Kup[24] = {0}, Fu[24] = {0};
  const double k = mat_K(m->mat_id, m->MC);
  double Dd[21], Dp[6];
  double B[6 * 24], S9[45], Om[6 * 9], B_NL[9 * 24];
  double Kuu[300];
  const double p_e = m->U[eeq(m, e + 1, HYDRO_PRESSURE) - 1];
  memset(Kuu, 0, sizeof(Kuu));
  for (int g = 0; g < 8; g++) {
    const double dWt = m->wts[g] * m->det[(size_t)e * 8 + g];
    const double* C = m->Cst + ((size_t)e * 8 + g) * 6;
    const double* G = m->NiXj + ((size_t)e * 8 + g) * 24;
    orc_material_D(m->mat_id, m->MC, C, p_e, Dd, Dp);
    double J = J_C(C);
    memset(B, 0, sizeof(B));
    memset(S9, 0, sizeof(S9));
    memset(Om, 0, sizeof(Om));
    memset(B_NL, 0, sizeof(B_NL));
    make_B_L(G, B);
    make_S9(m->S + ((size_t)e * 8 + g) * 6, S9);
    make_Omega(m->O + ((size_t)e * 8 + g) * 9, Om);
    make_B_NL(G, B_NL);
    k_matABprod(6, 9, 24, Om, B_NL, 2.0, B);
    k_matBTDBprod(6, 24, B, Dd, 0.5 * dWt, Kuu);
    k_matBTDBprod(9, 24, B_NL, S9, dWt, Kuu);
    k_matBTVprod(6, 24, B, m->S + ((size_t)e * 8 + g) * 6, -0.5 * dWt, Fu);
    k_matBTVprod(6, 24, B, Dp, 0.5 * dWt, Kup);
    Fp += -(J - 1 - p_e / k) * dWt;
    Kpp += -1.0 / k * dWt;
  }
  /* assemble3 (SOLID81.h:54-94) */
  const uint32_t* c = m->conn + (size_t)e * 8;
  const double* Kp = Kuu;
  int rc = 0;
  for (int i = 0; i < 8; i++)
    for (int di = 0; di < 3; di++)
      for (int j = i; j < 8; j++)
        for (int dj = 0; dj < 3; dj++) {
          if (i == j && dj < di) continue;
          rc |= add_value(m, neq(m, c[i], di), neq(m, c[j], dj), *Kp);
          Kp++;
        }
  const uint32_t elEq = eeq(m, e + 1, HYDRO_PRESSURE);
  for (int i = 0; i < 8; i++)
    for (int di = 0; di < 3; di++) rc |= add_value(m, neq(m, c[i], di), elEq, Kup[i * 3 + di]);
  rc |= add_value(m, elEq, elEq, Kpp);
  for (int i = 0; i < 8; i++)
    for (int di = 0; di < 3; di++) m->F[neq(m, c[i], di) - 1] += Fu[i * 3 + di];
  m->F[elEq - 1] += Fp;
  return rc;
}

/* ----------------------------------------------------------------------- */
/* TETRA0 (TETRA0.cpp)                                                      */
/* ----------------------------------------------------------------------- */

/* 4x4 determinant by partial-pivoting LU, the same algorithm as the oracle
 * build's dense-matrix shim (oracle/refshim/Eigen/Dense). */
static double det4_lu(const double* M) {
  double a[16];
  memcpy(a, M, sizeof(a));
  double det = 1.0;
  for (int k = 0; k < 4; k++) {
    int p = k;
    double best = fabs(a[k * 4 + k]);
    for (int i = k + 1; i < 4; i++) {
      double v = fabs(a[i * 4 + k]);
      if (v > best) { best = v; p = i; }
    }
    if (best == 0.0) return 0.0;
    if (p != k) {
      for (int j = 0; j < 4; j++) {
        double t = a[k * 4 + j];
        a[k * 4 + j] = a[p * 4 + j];
        a[p * 4 + j] = t;
      }
      det = -det;
    }
    const double piv = a[k * 4 + k];
    det *= piv;
    for (int i = k + 1; i < 4; i++) {
      const double f = a[i * 4 + k] / piv;
      for (int j = k + 1; j < 4; j++) a[i * 4 + j] -= f * a[k * 4 + j];
    }
  }
  return det;
}

/* the element strain matrix B (6x12, makeB TETRA0.cpp:110-184), the elastic
 * matrix C (packed MatSym<6>, makeC :186-199) and the volume (det[1 X] / 6) */
static void tetra0_B_C(const orc_model* m, uint32_t e, double* B, double* Cm,
                       double* vol_out) {
  const uint32_t* c = m->conn + (size_t)e * 4;
  const double* P[4];
  for (int a = 0; a < 4; a++) P[a] = m->xyz + (size_t)(c[a] - 1) * 3;
  double S[16];
  for (int a = 0; a < 4; a++) {
    S[a * 4 + 0] = 1.;
    S[a * 4 + 1] = P[a][0];
    S[a * 4 + 2] = P[a][1];
    S[a * 4 + 3] = P[a][2];
  }
  const double vol = det4_lu(S) / 6.;
  *vol_out = vol;
  memset(B, 0, sizeof(double) * 72);
  memset(Cm, 0, sizeof(double) * 21);
  /* makeC (TETRA0.cpp:186-199); MatSym<6>::comp index = 6*i - (i-1)*i/2 + (j-i) */
  const double E = m->eparams[EPAR * e], my = m->eparams[EPAR * e + 1];
  const double A = E / ((1. + my) * (1. - 2. * my));
#define CIDX(i, j) (6 * (i) - ((i) - 1) * (i) / 2 + ((j) - (i)))
  Cm[CIDX(0, 0)] = (1. - my) * A;
  Cm[CIDX(0, 1)] = my * A;
  Cm[CIDX(0, 2)] = my * A;
  Cm[CIDX(1, 1)] = (1. - my) * A;
  Cm[CIDX(1, 2)] = my * A;
  Cm[CIDX(2, 2)] = (1. - my) * A;
  Cm[CIDX(3, 3)] = (1. / 2. - my) * A;
  Cm[CIDX(4, 4)] = (1. / 2. - my) * A;
  Cm[CIDX(5, 5)] = (1. / 2. - my) * A;
#undef CIDX
  /* makeB (TETRA0.cpp:110-184) */
  const double x12 = P[0][0] - P[1][0], x13 = P[0][0] - P[2][0], x14 = P[0][0] - P[3][0];
  const double x23 = P[1][0] - P[2][0], x24 = P[1][0] - P[3][0], x34 = P[2][0] - P[3][0];
  const double x21 = -1. * x12, x31 = -1. * x13, x32 = -1. * x23, x42 = -1. * x24, x43 = -1. * x34;
  const double y12 = P[0][1] - P[1][1], y13 = P[0][1] - P[2][1], y14 = P[0][1] - P[3][1];
  const double y23 = P[1][1] - P[2][1], y24 = P[1][1] - P[3][1], y34 = P[2][1] - P[3][1];
  const double y21 = -1. * y12, y31 = -1. * y13, y32 = -1. * y23, y42 = -1. * y24, y43 = -1. * y34;
  const double z12 = P[0][2] - P[1][2], z13 = P[0][2] - P[2][2], z14 = P[0][2] - P[3][2];
  const double z23 = P[1][2] - P[2][2], z24 = P[1][2] - P[3][2], z34 = P[2][2] - P[3][2];
  const double z21 = -1. * z12, z31 = -1. * z13, z32 = -1. * z23, z42 = -1. * z24, z43 = -1. * z34;
  double b[4], cc[4], d[4];
  b[0] = y42 * z32 - y32 * z42;
  b[1] = y31 * z43 - y34 * z13;
  b[2] = y24 * z14 - y14 * z24;
  b[3] = y13 * z21 - y12 * z31;
  cc[0] = x32 * z42 - x42 * z32;
  cc[1] = x43 * z31 - x13 * z34;
  cc[2] = x14 * z24 - x24 * z14;
  cc[3] = x21 * z13 - x31 * z12;
  d[0] = x42 * y32 - x32 * y42;
  d[1] = x31 * y43 - x34 * y13;
  d[2] = x24 * y14 - x14 * y24;
  d[3] = x13 * y21 - x12 * y31;
  const double Af = -1. / 6. / vol;
  for (int i = 0; i < 4; i++) {
    B[0 + 3 * i] = b[i] * Af;
    B[13 + 3 * i] = cc[i] * Af;
    B[26 + 3 * i] = d[i] * Af;
    B[36 + 3 * i] = cc[i] * Af;
    B[37 + 3 * i] = b[i] * Af;
    B[49 + 3 * i] = d[i] * Af;
    B[50 + 3 * i] = cc[i] * Af;
    B[60 + 3 * i] = d[i] * Af;
    B[62 + 3 * i] = b[i] * Af;
  }
}

static int tetra0_buildK(orc_model* m, uint32_t e) {
  double Ke[78];
  memset(Ke, 0, sizeof(Ke));
  double B[6 * 12], Cm[21], vol;
  tetra0_B_C(m, e, B, Cm, &vol);
  const uint32_t* c = m->conn + (size_t)e * 4;
  k_matBTDBprod(6, 12, B, Cm, vol, Ke);
  /* Element::assembleK(Ke, {UX,UY,UZ}) (element.h:281-303) */
  const double* Kp = Ke;
  int rc = 0;
  for (int i = 0; i < 4; i++)
    for (int di = 0; di < 3; di++)
      for (int j = i; j < 4; j++)
        for (int dj = 0; dj < 3; dj++) {
          if (i == j && dj < di) continue;
          rc |= add_value(m, neq(m, c[i], di), neq(m, c[j], dj), *Kp);
          Kp++;
        }
  return rc;
}

/* ElementTETRA0::update (TETRA0.cpp:79-108): strains = -B U (matBVprod with
 * coefficient -1), stress = C strains (matBVprod of the MatSym C); out: six
 * stress components per element in the element's order (xx, yy, zz, xy, yz,
 * xz), from the model's current U. */
int orc_tetra0_stress(orc_model* m, double* out) {
  if (!m->setup_done || m->etype != ET_TETRA0) return fail(m, "tetra0_stress: a set-up TETRA0 model");
  for (uint32_t e = 0; e < m->n_elems; e++) {
    double B[72], Cm[21], vol, U[12], strain[6] = {0, 0, 0, 0, 0, 0}, C[36];
    tetra0_B_C(m, e, B, Cm, &vol);
    const uint32_t* c = m->conn + (size_t)e * 4;
    for (int a = 0; a < 4; a++)
      for (int d = 0; d < 3; d++) U[3 * a + d] = m->U[neq(m, c[a], d) - 1];
    for (int i = 0; i < 6; i++)
      for (int j = 0; j < 12; j++) strain[i] += B[i * 12 + j] * U[j] * -1.0;
    /* MatSym<6>::toMat: both triangles from the packed upper storage */
    for (int i = 0; i < 6; i++)
      for (int j = 0; j < 6; j++) {
        const int a = i < j ? i : j, b = i < j ? j : i;
        C[i * 6 + j] = Cm[6 * a - (a - 1) * a / 2 + (b - a)];
      }
    double* st = out + (size_t)e * 6;
    for (int i = 0; i < 6; i++) {
      st[i] = 0.0;
      for (int j = 0; j < 6; j++) st[i] += C[i * 6 + j] * strain[j] * 1.0;
    }
  }
  return 0;
}

/* ----------------------------------------------------------------------- */
/* QUADTH (QUADTH.cpp:22-67), SurfaceLINETH (QUADTH.cpp:70-121)           */
/* ----------------------------------------------------------------------- */

static int quadth_buildK(orc_model* m, uint32_t e) {
  double Ke[10];
  memset(Ke, 0, sizeof(Ke));
  double Fe[4] = {0, 0, 0, 0};
  const double kc = m->eparams[EPAR * e], vflux = m->eparams[EPAR * e + 1];
  const double matk[3] = {kc, 0.0, kc};
  for (int g = 0; g < 4; g++) {
    const double dWt = m->wts[g] * m->det[(size_t)e * 4 + g];
    const double* G = m->NiXj + ((size_t)e * 4 + g) * 8;
    const double Bm[8] = {G[0], G[2], G[4], G[6], G[1], G[3], G[5], G[7]};
    k_matBTDBprod(2, 4, Bm, matk, dWt, Ke);
    /* volume flux: Fe += N (volFlux dWt) */
    if (vflux != 0.0)
      for (int i = 0; i < 4; i++) Fe[i] += m->Nq[g * 4 + i] * (vflux * dWt);
  }
  const uint32_t* c = m->conn + (size_t)e * 4;
  const double* Kp = Ke;
  int rc = 0;
  for (int i = 0; i < 4; i++)
    for (int j = i; j < 4; j++) {
      rc |= add_value(m, neq(m, c[i], TEMP), neq(m, c[j], TEMP), *Kp);
      Kp++;
    }
  for (int i = 0; i < 4; i++) m->F[neq(m, c[i], TEMP) - 1] += Fe[i];
  return rc;
}

/* ElementQUADTH::buildC (QUADTH.cpp:51-67): Ce_ij += N_i N_j rho c dWt, then
 * Element::assembleC (element.h:306-329) in assembleK's upper-triangle order */
static int quadth_buildC(orc_model* m, uint32_t e) {
  double Ce[10];
  memset(Ce, 0, sizeof(Ce));
  const double rho = m->eparams[EPAR * e + 2], cap = m->eparams[EPAR * e + 3];
  for (int g = 0; g < 4; g++) {
    const double dWt = m->wts[g] * m->det[(size_t)e * 4 + g];
    const double* ff = m->Nq + g * 4;
    int k = 0;
    for (int i = 0; i < 4; i++)
      for (int j = i; j < 4; j++, k++) Ce[k] += ff[i] * ff[j] * rho * cap * dWt;
  }
  const uint32_t* c = m->conn + (size_t)e * 4;
  int rc = 0, k = 0;
  for (int i = 0; i < 4; i++)
    for (int j = i; j < 4; j++, k++)
      rc |= add_value_to(m, m->cval, neq(m, c[i], TEMP), neq(m, c[j], TEMP), Ce[k]);
  return rc;
}

/* SurfaceLINETH::buildK (QUADTH.cpp:86-121): 2-point Gauss (isoparametric.h:44-48),
 * dWt = w * |x2 - x1| / 2 (isoparametric.cpp:13-27, Vec::length).  The flux
 * loop runs before the convection loop; convection adds N N^T htc dWt to Ke
 * and (N N^T htc dWt) etemp to Fe term by term (matBVprod of a MatSym, Mat.h). */
static int line_buildK(orc_model* m, uint32_t l) {
  const uint32_t na = m->line_conn[2 * l], nb = m->line_conn[2 * l + 1];
  double q = 0.0;
  for (int d = 0; d < 3; d++) {
    const double dx = m->xyz[(size_t)(nb - 1) * 3 + d] - m->xyz[(size_t)(na - 1) * 3 + d];
    q += dx * dx;
  }
  const double det = sqrt(q) * 0.5;
  const double* par = m->line_par + 4 * (size_t)l;
  const double htc = par[0], flux = par[1], et[2] = {par[2], par[3]};
  double Ke[3] = {0.0, 0.0, 0.0}, Fe[2] = {0.0, 0.0};
  const double gr[2] = {-GP_A, GP_A};
  if (flux != 0.0)
    for (int g = 0; g < 2; g++) {
      const double dWt = 1.0 * det;
      const double Ns[2] = {0.5 * (1.0 - gr[g]), 0.5 * (1.0 + gr[g])};
      for (int i = 0; i < 2; i++) Fe[i] += Ns[i] * (flux * dWt);
    }
  if (htc != 0.0)
    for (int g = 0; g < 2; g++) {
      const double dWt = 1.0 * det;
      const double Ns[2] = {0.5 * (1.0 - gr[g]), 0.5 * (1.0 + gr[g])};
      const double t00 = Ns[0] * Ns[0] * htc * dWt, t01 = Ns[0] * Ns[1] * htc * dWt,
                   t11 = Ns[1] * Ns[1] * htc * dWt;
      Ke[0] += t00;
      Ke[1] += t01;
      Ke[2] += t11;
      const double T[2][2] = {{t00, t01}, {t01, t11}};
      for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) Fe[i] += T[i][j] * et[j] * 1.0;
    }
  int rc = add_value(m, neq(m, na, TEMP), neq(m, na, TEMP), Ke[0]);
  rc |= add_value(m, neq(m, na, TEMP), neq(m, nb, TEMP), Ke[1]);
  rc |= add_value(m, neq(m, nb, TEMP), neq(m, nb, TEMP), Ke[2]);
  m->F[neq(m, na, TEMP) - 1] += Fe[0];
  m->F[neq(m, nb, TEMP) - 1] += Fe[1];
  return rc;
}

/* ----------------------------------------------------------------------- */
/* PLANE41 (PLANE41.cpp): 4-node plane-strain u/p quad, Mat operator algebra */
/* ----------------------------------------------------------------------- */

/* Mat::operator*(Mat) (Mat.h:198-212): element = 0, += a_il b_lj in l order */
static void mat_mul(const double* A, int M, int N, const double* B, int K, double* out) {
  for (int i = 0; i < M; i++)
    for (int j = 0; j < K; j++) {
      double el = 0.0;
      for (int l = 0; l < N; l++) el += A[i * N + l] * B[l * K + j];
      out[i * K + j] = el;
    }
}

static void mat_T(const double* A, int M, int N, double* out) {
  for (int i = 0; i < M; i++)
    for (int j = 0; j < N; j++) out[j * M + i] = A[i * N + j];
}

/* components of PLANE41 (PLANE41.cpp:11): M_XX, M_YY, M_XY */
static const int P41_COMPS[3] = {M_XX, M_YY, M_XY};

static void plane41_B(const double* G, double* B /*3x8*/, double* Bw /*4x8*/) {
  /* make_B, make_Bomega (PLANE41.cpp:103-118); G[2a+d] = dN_a/dx_d */
  memset(B, 0, sizeof(double) * 24);
  memset(Bw, 0, sizeof(double) * 32);
  for (int a = 0; a < 4; a++) {
    const double gx = G[2 * a], gy = G[2 * a + 1];
    B[0 * 8 + 2 * a] = gx;
    B[1 * 8 + 2 * a + 1] = gy;
    B[2 * 8 + 2 * a] = gy;
    B[2 * 8 + 2 * a + 1] = gx;
    Bw[0 * 8 + 2 * a] = gx;
    Bw[1 * 8 + 2 * a] = gy;
    Bw[2 * 8 + 2 * a + 1] = gx;
    Bw[3 * 8 + 2 * a + 1] = gy;
  }
}

/* ElementPLANE41::update (PLANE41.cpp:120-146) */
static void plane41_update(orc_model* m, uint32_t e) {
  const uint32_t* c = m->conn + (size_t)e * 4;
  double U[8];
  for (int a = 0; a < 4; a++) {
    U[2 * a] = m->U[neq(m, c[a], UX) - 1];
    U[2 * a + 1] = m->U[neq(m, c[a], UY) - 1];
  }
  const double p_e = m->U[eeq(m, e + 1, HYDRO_PRESSURE) - 1];
  for (int g = 0; g < 4; g++) {
    double B[24], Bw[32];
    plane41_B(m->NiXj + ((size_t)e * 4 + g) * 8, B, Bw);
    double* O = m->O + ((size_t)e * 4 + g) * 4;
    double* C = m->Cst + ((size_t)e * 4 + g) * 3;
    mat_mul(Bw, 4, 8, U, 1, O);
    C[0] = 1.0 + 2 * O[0] + 1.0 * (O[0] * O[0] + O[2] * O[2]);
    C[1] = 1.0 + 2 * O[3] + 1.0 * (O[3] * O[3] + O[1] * O[1]);
    C[2] = O[1] + O[2] + O[0] * O[1] + O[2] * O[3];
    double CV[6] = {C[0], C[2], 0.0, C[1], 0.0, 1.0};
    double S6[6];
    orc_material_S(m->mat_id, m->MC, CV, p_e, S6);
    double* S = m->S + ((size_t)e * 4 + g) * 3;
    for (int i = 0; i < 3; i++) S[i] = S6[P41_COMPS[i]];
  }
}

/* ElementPLANE41::buildK (PLANE41.cpp:31-101) and its assembleK (PLANE41.h:54-95) */
static int plane41_buildK(orc_model* m, uint32_t e) {
  double Kuu[64], Kup[8], Qe[8];
  memset(Kuu, 0, sizeof(Kuu));
  memset(Kup, 0, sizeof(Kup));
  memset(Qe, 0, sizeof(Qe));
  double Kpp = 0.0, Fp = 0.0;
  const double p_e = m->U[eeq(m, e + 1, HYDRO_PRESSURE) - 1];
  const double k = mat_K(m->mat_id, m->MC);
  for (int g = 0; g < 4; g++) {
    const double dWt = m->wts[g] * m->det[(size_t)e * 4 + g];
    const double* Cg = m->Cst + ((size_t)e * 4 + g) * 3;
    const double* S = m->S + ((size_t)e * 4 + g) * 3;
    const double* O = m->O + ((size_t)e * 4 + g) * 4;
    double CV[6] = {Cg[0], Cg[2], 0.0, Cg[1], 0.0, 1.0};
    double Dd[6], Dp[3];
    material_D_comps(m->mat_id, m->MC, 3, P41_COMPS, CV, p_e, Dd, Dp);
    const double Ec[9] = {Dd[0], Dd[1], Dd[2], Dd[1], Dd[3], Dd[4], Dd[2], Dd[4], Dd[5]};
    double IC[3];
    IC_C(CV, IC);
    const double J = IC[2];
    double B[24], Bw[32];
    plane41_B(m->NiXj + ((size_t)e * 4 + g) * 8, B, Bw);
    const double S4[16] = {S[0], S[2], 0.0, 0.0, S[2], S[1], 0.0, 0.0,
                           0.0, 0.0, S[0], S[2], 0.0, 0.0, S[2], S[1]};
    const double Om[12] = {O[0], 0.0, O[2], 0.0, 0.0, O[1], 0.0, O[3], O[1], O[0], O[3], O[2]};
    double Bl[24];
    mat_mul(Om, 3, 4, Bw, 8, Bl);
    for (int i = 0; i < 24; i++) B[i] += Bl[i];
    double BT[24], BwT[32], t1[24], t2[64], t3[32], t4[64];
    mat_T(B, 3, 8, BT);
    mat_T(Bw, 4, 8, BwT);
    mat_mul(BT, 8, 3, Ec, 3, t1);   /* B^T E */
    mat_mul(t1, 8, 3, B, 8, t2);    /* (B^T E) B */
    mat_mul(BwT, 8, 4, S4, 4, t3);  /* Bw^T S */
    mat_mul(t3, 8, 4, Bw, 8, t4);   /* (Bw^T S) Bw */
    for (int i = 0; i < 64; i++) Kuu[i] += (t2[i] * 2.0 + t4[i]) * dWt;
    Fp += (J - 1 - p_e / k) * dWt;
    double q[8];
    mat_mul(BT, 8, 3, S, 1, q);     /* B^T S (Mat * Vec) */
    for (int i = 0; i < 8; i++) Qe[i] += q[i] * dWt;
    double kup[8];
    mat_mul(BT, 8, 3, Dp, 1, kup);
    for (int i = 0; i < 8; i++) Kup[i] += kup[i] * dWt;
    Kpp -= 1.0 / k * dWt;
  }
  const uint32_t* c = m->conn + (size_t)e * 4;
  const uint32_t pe = eeq(m, e + 1, HYDRO_PRESSURE);
  const int dofs[2] = {UX, UY};
  int rc = 0;
  for (int i = 0; i < 4; i++)
    for (int j = i; j < 4; j++)
      for (int di = 0; di < 2; di++)
        for (int dj = 0; dj < 2; dj++) {
          if (i == j && dj > di) continue;
          rc |= add_value(m, neq(m, c[i], dofs[di]), neq(m, c[j], dofs[dj]),
                          Kuu[(i * 2 + di) * 8 + j * 2 + dj]);
        }
  for (int i = 0; i < 4; i++)
    for (int di = 0; di < 2; di++) rc |= add_value(m, neq(m, c[i], dofs[di]), pe, Kup[i * 2 + di]);
  rc |= add_value(m, pe, pe, Kpp);
  for (int i = 0; i < 4; i++)
    for (int di = 0; di < 2; di++) m->F[neq(m, c[i], dofs[di]) - 1] += -Qe[i * 2 + di];
  m->F[pe - 1] += -Fp;
  return rc;
}

/* ----------------------------------------------------------------------- */
/* RigidBodyMpc::update (Mpc.cpp:70-164)                                    */
/* ----------------------------------------------------------------------- */

static const int LC[3][3][3] = {{{0, 0, 0}, {0, 0, 1}, {0, -1, 0}},
                                {{0, 0, -1}, {0, 0, 0}, {1, 0, 0}},
                                {{0, 1, 0}, {-1, 0, 0}, {0, 0, 0}}};
static const int I3[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};

static void rigid_body_update(orc_model* m, rigid_body* rb) {
  double theta0[3], w0[3];
  theta0[0] = m->U[neq(m, rb->master, ROTX) - 1];
  theta0[1] = m->U[neq(m, rb->master, ROTY) - 1];
  theta0[2] = m->U[neq(m, rb->master, ROTZ) - 1];
  w0[0] = m->U[neq(m, rb->master, UX) - 1];
  w0[1] = m->U[neq(m, rb->master, UY) - 1];
  w0[2] = m->U[neq(m, rb->master, UZ) - 1];
  double q = 0;
  for (int i = 0; i < 3; i++) q += theta0[i] * theta0[i];
  const double thetaNorm = sqrt(q);
  double c1, c2, c3, c4;
  if (thetaNorm < 1.0e-3) {
    c1 = 1.0;
    c2 = 0.5;
    c3 = -1.0 / 3.0;
    c4 = -1.0 / 12.0;
  } else {
    c1 = sin(thetaNorm) / thetaNorm;
    c2 = (1.0 - cos(thetaNorm)) / (thetaNorm * thetaNorm);
    c3 = (thetaNorm * cos(thetaNorm) - sin(thetaNorm)) / (thetaNorm * thetaNorm * thetaNorm);
    c4 = (thetaNorm * sin(thetaNorm) - 2.0 + 2.0 * cos(thetaNorm)) /
         (thetaNorm * thetaNorm * thetaNorm * thetaNorm);
  }
  double C[3][3];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) {
      double tm = LC[i][0][j] * theta0[0] + LC[i][1][j] * theta0[1] + LC[i][2][j] * theta0[2];
      C[i][j] = cos(thetaNorm) * I3[i][j] + c1 * tm + c2 * theta0[i] * theta0[j];
    }
  const double* mp = m->xyz + (size_t)(rb->master - 1) * 3;
  for (uint32_t n = 0; n < rb->n_slaves; n++) {
    const double* sp = m->xyz + (size_t)(rb->slaves[n] - 1) * 3;
    double pq[3] = {sp[0] - mp[0], sp[1] - mp[1], sp[2] - mp[2]};
    for (uint32_t d = 0; d < rb->n_dofs; d++) {
      const int i = rb->dofs[d];
      double cD[3][3];
      for (int j = 0; j < 3; j++)
        for (int l = 0; l < 3; l++)
          cD[j][l] = I3[i][j] * (-c1) * theta0[l] +
                     c3 * theta0[l] *
                         (LC[i][0][j] * theta0[0] + LC[i][1][j] * theta0[1] +
                          LC[i][2][j] * theta0[2]) +
                     c1 * LC[i][l][j] + c4 * theta0[l] * theta0[i] * theta0[j] +
                     c2 * (I3[i][l] * theta0[j] + theta0[i] * I3[j][l]);
      mpc_eq* q2 = &m->mpcs[rb->first_mpc + n * rb->n_dofs + d];
      q2->b = w0[i] + (C[i][0] - I3[i][0]) * pq[0] + (C[i][1] - I3[i][1]) * pq[1] +
              (C[i][2] - I3[i][2]) * pq[2] - m->U[neq(m, rb->slaves[n], rb->dofs[d]) - 1];
      q2->t[2].coef = -(cD[0][0] * pq[0] + cD[1][0] * pq[1] + cD[2][0] * pq[2]);
      q2->t[3].coef = -(cD[0][1] * pq[0] + cD[1][1] * pq[1] + cD[2][1] * pq[2]);
      q2->t[4].coef = -(cD[0][2] * pq[0] + cD[1][2] * pq[1] + cD[2][2] * pq[2]);
    }
  }
}

/* ----------------------------------------------------------------------- */
/* FEStorage::updateResults / assembleGlobalEqMatrices                      */
/* ----------------------------------------------------------------------- */

int orc_update(orc_model* m) {
  if (!m->setup_done) return fail(m, "setup first");
  if (m->etype == ET_SOLID81)
    for (uint32_t e = 0; e < m->n_elems; e++) solid81_update(m, e);
  else if (m->etype == ET_PLANE41)
    for (uint32_t e = 0; e < m->n_elems; e++) plane41_update(m, e);
  return 0;
}

int orc_assemble(orc_model* m) {
  if (!m->setup_done) return fail(m, "setup first");
  for (int b = 0; b < 3; b++)
    if (m->blk[b].nnz) memset(m->blk[b].values, 0, sizeof(double) * m->blk[b].nnz);
  memset(m->F, 0, sizeof(double) * (m->n_dofs + m->n_mpc));
  int rc = 0;
  for (uint32_t e = 0; e < m->n_elems && !rc; e++) {
    if (m->etype == ET_SOLID81)
      rc |= solid81_buildK(m, e);
    else if (m->etype == ET_TETRA0)
      rc |= tetra0_buildK(m, e);
    else if (m->etype == ET_PLANE41)
      rc |= plane41_buildK(m, e);
    else
      rc |= quadth_buildK(m, e);
  }
  for (uint32_t l = 0; l < m->n_lines && !rc; l++) rc |= line_buildK(m, l);
  if (rc) return 1;
  for (uint32_t r = 0; r < m->n_rbs; r++) rigid_body_update(m, &m->rbs[r]);
  for (uint32_t k = 0; k < m->n_lmpc; k++) {
    m->F[m->lm_eq[k] - 1] = m->lm_b[k];
    for (uint32_t t = m->lm_ptr[k]; t < m->lm_ptr[k + 1]; t++)
      rc |= add_value(m, m->lm_eq[k], neq(m, m->lm_node[t], m->lm_dof[t]), m->lm_coef[t]);
  }
  for (uint32_t k = 0; k < m->n_rmpc; k++) {
    mpc_eq* q = &m->mpcs[k];
    m->F[q->eq - 1] = q->b;
    for (int t = 0; t < 5; t++) rc |= add_value(m, q->eq, neq(m, q->t[t].node, q->t[t].dof), q->t[t].coef);
  }
  /* transient: zeroC, zeroM, buildC / buildM over the elements (FEStorage.cpp:63-76);
   * SurfaceLINETH and buildM of QUADTH add nothing (QUADTH.h:25, :48-49) */
  if (m->transient && !rc) {
    for (int b = 0; b < 3; b++)
      if (m->blk[b].nnz) {
        memset(m->cval[b], 0, sizeof(double) * m->blk[b].nnz);
        memset(m->mval[b], 0, sizeof(double) * m->blk[b].nnz);
      }
    for (uint32_t e = 0; e < m->n_elems && !rc; e++) rc |= quadth_buildC(m, e);
  }
  return rc;
}

int orc_add_surface_lines(orc_model* m, uint32_t n, const uint32_t* conn, const double* htc,
                          const double* flux, const double* etemp) {
  if (m->setup_done) return fail(m, "add_surface_lines after setup");
  if (m->etype != ET_QUADTH) return fail(m, "surface lines need a QUADTH model");
  const uint32_t L = m->n_lines + n;
  m->line_conn = (uint32_t*)realloc(m->line_conn, sizeof(uint32_t) * 2 * (L ? L : 1));
  m->line_par = (double*)realloc(m->line_par, sizeof(double) * 4 * (L ? L : 1));
  for (uint32_t i = 0; i < n; i++) {
    const uint32_t l = m->n_lines + i;
    m->line_conn[2 * l] = conn[2 * i];
    m->line_conn[2 * l + 1] = conn[2 * i + 1];
    m->line_par[4 * l + 0] = htc ? htc[i] : 0.0;
    m->line_par[4 * l + 1] = flux ? flux[i] : 0.0;
    m->line_par[4 * l + 2] = etemp ? etemp[2 * i] : 0.0;
    m->line_par[4 * l + 3] = etemp ? etemp[2 * i + 1] : 0.0;
  }
  m->n_lines = L;
  return 0;
}

int orc_set_transient(orc_model* m, int on) {
  if (m->setup_done) return fail(m, "set_transient after setup");
  m->transient = on != 0;
  return 0;
}

static int get_cm(orc_model* m, double** vals, int block, double* values) {
  if (!m->setup_done || !m->transient) return fail(m, "C, M: not a transient model");
  const int b = slot_of(block);
  if (m->blk[b].nnz) memcpy(values, vals[b], sizeof(double) * m->blk[b].nnz);
  return 0;
}

int orc_get_C(orc_model* m, int block, double* values) { return get_cm(m, m->cval, block, values); }
int orc_get_M(orc_model* m, int block, double* values) { return get_cm(m, m->mval, block, values); }

int orc_get_K(orc_model* m, int block, double* values) {
  csr_block* b = &m->blk[slot_of(block)];
  if (b->nnz) memcpy(values, b->values, sizeof(double) * b->nnz);
  return 0;
}

/* matBVprod(SparseSymMatrix&) SparseMatrix.cpp:497-519, matBVprod(SparseMatrix&)
 * :522-540, matBTVprod(SparseMatrix&) :542-558 */
int orc_block_mv(orc_model* m, int block, int trans, const double* x, double coef, double* y) {
  const csr_block* b = &m->blk[slot_of(block)];
  const double eps = 1e-20;
  if (block == 1 || block == 2) {
    /* The reference walks j = 1..n for every row i through value(), which
     * returns 0 for a structural zero.  Walking only the stored entries in
     * the same order (column i of the upper triangle by ascending row, then
     * row i right of the diagonal) gives the same sums, except that the
     * reference also adds +-0 for each structural zero, which can only change
     * the sign of a zero result; it costs O(nnz) instead of O(n^2 log). */
    const uint32_t n = b->rows;
    uint32_t* cp = (uint32_t*)calloc((size_t)n + 1, sizeof(uint32_t));
    uint32_t* cr = (uint32_t*)malloc(sizeof(uint32_t) * (b->nnz ? b->nnz : 1));
    uint32_t* ck = (uint32_t*)malloc(sizeof(uint32_t) * (b->nnz ? b->nnz : 1));
    for (uint32_t k = 0; k < b->nnz; k++) cp[b->columns[k]]++;
    for (uint32_t i = 0; i < n; i++) cp[i + 1] += cp[i];
    uint32_t* pos = (uint32_t*)malloc(sizeof(uint32_t) * ((size_t)n + 1));
    memcpy(pos, cp, sizeof(uint32_t) * ((size_t)n + 1));
    for (uint32_t r = 1; r <= n; r++)
      for (uint32_t k = b->iofeir[r - 1] - 1; k < b->iofeir[r] - 1; k++) {
        const uint32_t c = b->columns[k];
        cr[pos[c - 1]] = r;
        ck[pos[c - 1]++] = k;
      }
    for (uint32_t i = 1; i <= n; i++) {
      for (uint32_t q = cp[i - 1]; q < cp[i]; q++) {   /* j = cr[q] <= i ascending */
        const uint32_t j = cr[q];
        if (fabs(x[j - 1]) > eps) y[i - 1] += b->values[ck[q]] * x[j - 1] * coef;
      }
      for (uint32_t k = b->iofeir[i - 1] - 1; k < b->iofeir[i] - 1; k++) {
        const uint32_t j = b->columns[k];
        if (j > i && fabs(x[j - 1]) > eps) y[i - 1] += b->values[k] * x[j - 1] * coef;
      }
    }
    free(cp); free(cr); free(ck); free(pos);
    return 0;
  }
  for (uint32_t i = 1; i <= b->rows; i++) {
    if (b->iofeir[i] - b->iofeir[i - 1] == 0) continue;
    const uint32_t st = b->iofeir[i - 1] - 1, en = b->iofeir[i] - 2;
    for (uint32_t j = st; j <= en; j++) {
      if (trans)
        y[b->columns[j] - 1] += b->values[j] * x[i - 1] * coef;
      else
        y[i - 1] += b->values[j] * x[b->columns[j] - 1] * coef;
    }
  }
  return 0;
}

int orc_get_F(orc_model* m, double* F) {
  memcpy(F, m->F, sizeof(double) * (m->n_dofs + m->n_mpc));
  return 0;
}
