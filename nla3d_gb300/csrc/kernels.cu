// Assembly kernels for sm_103a: SOLID81 (FP64 and mixed), its Jacobian
// precompute, TETRA0 / QUADTH, the fixed-order CSR gather and the rigid-body
// MPC rows.
//
// SOLID81 algebra (reference: SOLID81.cpp:29-82, 85-115):
//   B = 2 (B_L + Omega B_NL) is 2 * Bh, where for node a, displacement
//   component i and Voigt row (jk):  Bh[(jk)][i] = F_ij G_ak + F_ik G_aj
//   (j != k), F_ij G_aj (j == k);  F = I + O, G_a = dN_a/dX.
//   Kuu(a,i; b,k) += w * (Bh_a^T Dd' Bh_b)[i][k] + w * delta_ik G_a . S G_b
//       with Dd' = 2 * Dd (the reference halves Dd, materials_hyperelastic.cpp:124,
//       and scales B^T Dd B by w/2 with B = 2 Bh);
//   Fu_a   += -w * (F S G_a)              ( = -w/2 B^T S,  SOLID81.cpp:73 )
//   Kup_a  +=  w * (cof(F) G_a)           ( = w/2 B^T J C^-1, since J F C^-1 = cof F )
//   Fp     += -(J - 1 - p/k) w ;  Kpp += -w / k
// Writing Bh out, both Kuu terms are one contraction with a symmetric 9x9
// tensor per Gauss point:
//   Kuu(a,i; b,k) += sum_{L,N} G_aL A[iL][kN] G_bN,
//   A[iL][kN] = sum_{J,M} F_iJ wDd'[(JL)][(MN)] F_kM + delta_ik w S_LN,
// so one Gauss point costs 45 entries of A (about 300 FMA), h_a[ik] = A^T G_a
// per node and 3 FMA per Kuu entry, instead of 6 + the geometric term per
// entry and D Bh per node.  Since A is symmetric, K(a,i; b,k) = h_b[ki] . G_a
// as well, so h is formed only for i <= k (6 of the 9 blocks, 54 FMA per
// node) and the entries with i > k (off-diagonal node blocks only) read
// h_b[ki] and G_a.  These are the reference's products with the
// structural zeros of B, B_NL and Omega removed and the sums regrouped; they
// agree with the reference to rounding (the tests bound the difference at
// 1e-12 relative).
#include <atomic>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <type_traits>

#include "kernels.cuh"

namespace nla3d_gpu {

namespace {

constexpr int kWarpsPerBlock = 4;  // default launch shape
constexpr int kEPW = 4;                              // elements per warp
constexpr int kKuuPerElem = 300;
constexpr int kOwned = (kEPW * kKuuPerElem + 31) / 32;  // Kuu entries per lane (38)
constexpr double kGaussA = 0.5773502691896258;        // isoparametric.h:127

// Kuu entry t (assemble3 order, SOLID81.h:62-74) -> (a, i, b, k) packed.
__constant__ uchar4 c_kuu_entry[kKuuPerElem];

// FP64 kernel: the shape gradients of an element sum to zero at every Gauss
// point (sum_b G_b = J^-1 sum_b dN_b/dxi = 0), so K(a,i; 7,k) = sum_g h_a . G_7
// = -sum_{b<7} K(a,i; b,k), and likewise h_7 = -sum_{a<7} h_a.  The 63
// entries of node 7's column (a < 7, all nine (i,k)) are formed from the
// accumulated ones after the Gauss-point loop (7 adds each, in a fixed
// order), and then the 6 of node 7's own block, K(7,i; 7,k) = -sum_{a<7}
// K(a,i; 7,k), from those: 231 of the 300 entries take 24 FMAs each inside
// the loop, the minimum for blocks whose rows and columns sum to zero.  The
// formed entries differ from the direct sums by rounding only
// (|sum_b G_b| ~ eps |G|).
constexpr int kKuuColumn = 63;                                       // first pass
constexpr int kKuuCorner = 6;                                        // second pass
constexpr int kKuuDerived = kKuuColumn + kKuuCorner;                 // 69
constexpr int kKuuOwned = kKuuPerElem - kKuuDerived;                 // 231
constexpr int kOwned64 = (kEPW * kKuuOwned + 31) / 32;               // per lane (29)
// FP64 kernel block header: ownership words, stage positions, derived table
constexpr size_t kHead64Bytes =
    (sizeof(uint32_t) * kOwned64 * 32 + sizeof(uint16_t) * kOwned64 * 32 +
     sizeof(uint16_t) * kKuuDerived * 8 + 15) / 16 * 16;
__constant__ uint16_t c_kuu_owned[kKuuOwned];            // owned m -> assemble3 t
__constant__ uint16_t c_kuu_derived[kKuuDerived * 8];    // target t, then its 7 sources

// Mixed kernel: position in assemble3 order of the Kuu entry that
// D[(i,k), a, b] = sum h_a[ik] . G_b (i <= k) stands for, at [(a * 6 +
// hblock(i,k)) * 8 + b]: K(a,i; b,k) when a <= b, K(b,k; a,i) when a > b;
// 0xFFFF where a > b and i == k (the same entry as D[(i,i), b, a]).
constexpr int kDpos = 8 * 6 * 8;
constexpr size_t kDposBytes = kDpos * sizeof(uint16_t);
__constant__ uint16_t c_dpos[kDpos];

// -w F S: FP64, or a float pair (hi, lo) in the mixed kernel
template <typename TT>
struct ResidualType {
  using type = double;
};
template <>
struct ResidualType<float> {
  using type = float2;
};

// FP64 kernel: stride of one (i, k) block of h (3 N x 32 slots) in the warp
// scratch.
constexpr int kHStride = 96;

// the (i, k) blocks of h that are formed: i <= k, packed (6 blocks)
__host__ __device__ constexpr int hblock(int i, int k) {  // i <= k
  return 3 * i - (i * (i - 1)) / 2 + (k - i);
}

template <typename TT>
struct WarpSmem {
  typename ResidualType<TT>::type wP[9][32];  // per (element q, Gauss point g): -w F S
  TT wCof[9][32];      //  w cof(F)
  TT A[45][32];        //  symmetric 9x9 tangent tensor A[iL][kN], packed upper
  TT H[6 * kHStride];  // per (element q, node a) at the current Gauss point:
                       //  h_a[ik][N], i <= k, at hblock(i,k) * kHStride + 32 N + slot
  TT G[3][32];         //  G_a
};

// Mixed kernel: -w F S (float pairs) and w cof F (FP64: the pressure
// coupling K_up keeps FP64) are only needed between phase 1 and the residual
// / coupling pass that precedes the Gauss point loop, so they share their
// bytes with the staging buffer of the Kuu write after that loop.  Per
// (element q, Gauss point g) they sit at slot g * 4 + q, so the pass's
// broadcast reads of one Gauss point hit four consecutive words.  h stays in
// registers (each lane keeps its own node's).
template <>
struct WarpSmem<float> {
  float A[45][32];
  union {
    float stage[4 * 300];   // the quad's Kuu entries in assemble3 order, for the write
    struct {
      float2 wP[9][32];     // -w F S, float pairs
      double wCof[9][32];   // w cof F, FP64
      float wCofF[9][32];   // the same from the float F (for G's low part)
    };
  };
  float G[3][32];
};

__device__ __forceinline__ int sym6(int r, int s) {  // packed upper index, r <= s
  return 6 * r - ((r - 1) * r) / 2 + (s - r);
}

__device__ __forceinline__ int sym6u(int r, int s) { return r <= s ? sym6(r, s) : sym6(s, r); }

__device__ __forceinline__ int sym9(int p, int c) {  // packed upper 9x9, any order
  return p <= c ? 9 * p - ((p - 1) * p) / 2 + (c - p) : 9 * c - ((c - 1) * c) / 2 + (p - c);
}

// Voigt index of the symmetric pair (J, L): xx xy xz yy yz zz
__device__ __forceinline__ int voigt(int J, int L) {
  return J == L ? (J == 0 ? 0 : (J == 1 ? 3 : 5)) : (J + L == 1 ? 1 : (J + L == 2 ? 2 : 4));
}

__device__ __forceinline__ void flag_element(ElementStatus* st, uint32_t el1) {
  atomicAdd(&st->count, 1u);
  atomicMin(&st->first, el1);
}

template <typename TT>
__device__ __forceinline__ void tangent_from_coefficients(const TT At[6], const TT Bt[6],
                                                          const TT Ct[6], TT wk11, TT wk1,
                                                          TT wk2, TT wc0, TT sIIt, TT sI,
                                                          TT wD[21]);

// Material response at one Gauss point (materials_hyperelastic.cpp:30-129).
// Inputs: C (Voigt), p_state (for S), p_cur (for Dd).  Outputs: S, J and the
// coefficient form of w*2*Dd:
//   wD = A (x) P + B (x) Q + Ci (x) R + sIIt * IIt + sI * (I (x) I - II)
template <typename TT>
struct MatOut {
  double S[6];
  double J;
};

template <typename TT>
__device__ __forceinline__ void material(int mat_id, const double* mc, const double C[6],
                                         double p_state, double p_cur, double w, MatOut<TT>& o,
                                         TT wD[21]) {
  const double I1 = C[0] + C[3] + C[5];
  const double I2 = C[0] * C[3] + C[3] * C[5] + C[0] * C[5] - C[1] * C[1] - C[4] * C[4] -
                    C[2] * C[2];
  const double detC = C[0] * (C[3] * C[5] - C[4] * C[4]) - C[1] * (C[1] * C[5] - C[4] * C[2]) +
                      C[2] * (C[1] * C[4] - C[3] * C[2]);
  const double J = sqrt(detC);
  const double rc = rcbrt(J);
  const double pp = rc * rc;       // J^(-2/3)
  const double pppp = pp * pp;     // J^(-4/3)
  const double oo = 1.0 / (J * J);
  double Ci[6];
  Ci[0] = oo * (C[3] * C[5] - C[4] * C[4]);
  Ci[1] = oo * (C[2] * C[4] - C[1] * C[5]);
  Ci[2] = oo * (C[1] * C[4] - C[2] * C[3]);
  Ci[3] = oo * (C[0] * C[5] - C[2] * C[2]);
  Ci[4] = oo * (C[1] * C[2] - C[0] * C[4]);
  Ci[5] = oo * (C[0] * C[3] - C[1] * C[1]);
  const double t13 = (1.0 / 3.0) * I1, t23 = (2.0 / 3.0) * I2;
  // W derivatives at (I1 J^-2/3, I2 J^-4/3) (materials_hyperelastic.cpp:135-204)
  double a1, a2 = 0.0, a11 = 0.0;
  if (mat_id == 1) {
    a1 = 0.5 * mc[0];
  } else if (mat_id == 2) {
    const double d = I1 * pp - 3.0;
    a1 = mc[0] + 2 * mc[1] * d + 3 * mc[2] * d * d;
    a2 = mc[3];
    a11 = 2 * mc[1] + 6 * mc[2] * d;
  } else {
    a1 = mc[0];
    a2 = mc[1];
  }
  const double I6[6] = {1.0, 0.0, 0.0, 1.0, 0.0, 1.0};
  double A[6], B[6];
#pragma unroll
  for (int i = 0; i < 6; i++) {
    A[i] = I6[i] - t13 * Ci[i];
    B[i] = I1 * I6[i] - C[i] - t23 * Ci[i];
  }
  const double ko1 = 2 * a1 * pp, ko2 = 2 * a2 * pppp, pJs = p_state * J;
#pragma unroll
  for (int i = 0; i < 6; i++) o.S[i] = ko1 * A[i] + ko2 * B[i] + pJs * Ci[i];
  o.J = J;
  // tangent coefficients (Dd before the reference's /2, times w)
  const double k11 = 4.0 * a11 * pppp, k1 = (4.0 / 3.0) * a1 * pp, k2 = (8.0 / 3.0) * a2 * pppp;
  const double pj = p_cur * J;
  const double c0 = pj - k1 * t13 - k2 * t23;
  const TT sIIt = (TT)(w * (2.0 * pj - k1 * I1 - k2 * I2));
  const TT sI = (TT)(w * 1.5 * k2);
  // scalar coefficients in FP64, the 6-vectors P, Q, R in the tangent type
  const TT wk11 = (TT)(w * k11), wk1 = (TT)(w * k1), wk2 = (TT)(w * k2), wc0 = (TT)(w * c0);
  TT At[6], Bt[6], Ct[6];
#pragma unroll
  for (int i = 0; i < 6; i++) {
    At[i] = (TT)A[i];
    Bt[i] = (TT)B[i];
    Ct[i] = (TT)Ci[i];
  }
  tangent_from_coefficients<TT>(At, Bt, Ct, wk11, wk1, wk2, wc0, sIIt, sI, wD);
}

// w * 2 Dd, packed upper Voigt, from the coefficient form
//   A (x) P + B (x) Q + Ci (x) R + sIIt * IIt + sI * (I (x) I - II)
// with P = wk11 A - wk1 Ci, Q = -wk2 Ci, R = -wk1 A - wk2 B + wc0 Ci
// (materials_hyperelastic.cpp:64-129 with the reference's /2 taken out).
template <typename TT>
__device__ __forceinline__ void tangent_from_coefficients(const TT At[6], const TT Bt[6],
                                                          const TT Ct[6], TT wk11, TT wk1,
                                                          TT wk2, TT wc0, TT sIIt, TT sI,
                                                          TT wD[21]) {
  TT P[6], Q[6], R[6];
#pragma unroll
  for (int i = 0; i < 6; i++) {
    P[i] = wk11 * At[i] - wk1 * Ct[i];
    Q[i] = -wk2 * Ct[i];
    R[i] = -wk1 * At[i] - wk2 * Bt[i] + wc0 * Ct[i];
  }
  // IIt (materials_hyperelastic.cpp:97-108): -sym(Ci (x) Ci), packed upper
  const TT c_xx = Ct[0], c_xy = Ct[1], c_xz = Ct[2], c_yy = Ct[3], c_yz = Ct[4], c_zz = Ct[5];
  const TT h = (TT)0.5;
  const TT IIt[21] = {
      -c_xx * c_xx, -c_xx * c_xy, -c_xx * c_xz, -c_xy * c_xy, -c_xy * c_xz, -c_xz * c_xz,
      -h * (c_xx * c_yy + c_xy * c_xy), -h * (c_xx * c_yz + c_xz * c_xy), -c_xy * c_yy,
      -h * (c_xy * c_yz + c_xz * c_yy), -c_xz * c_yz,
      -h * (c_xx * c_zz + c_xz * c_xz), -c_xy * c_yz, -h * (c_xy * c_zz + c_xz * c_yz),
      -c_xz * c_zz,
      -c_yy * c_yy, -c_yy * c_yz, -c_yz * c_yz,
      -h * (c_yy * c_zz + c_yz * c_yz), -c_yz * c_zz,
      -c_zz * c_zz};
  // I (x) I - II, packed upper: +1 at (0,3),(0,5),(3,5); -1/2 at (1,1),(2,2),(4,4)
  int idx = 0;
#pragma unroll
  for (int r = 0; r < 6; r++)
#pragma unroll
    for (int s = r; s < 6; s++, idx++) {
      TT v = At[r] * P[s] + Bt[r] * Q[s] + Ct[r] * R[s] + sIIt * IIt[idx];
      const bool plus = (r == 0 && (s == 3 || s == 5)) || (r == 3 && s == 5);
      const bool minus = (r == s) && (r == 1 || r == 2 || r == 4);
      if (plus) v += sI;
      if (minus) v -= h * sI;
      wD[idx] = v;
    }
}

// ---------------------------------------------------------------------------
// Float-pair ("double-word") arithmetic for the mixed path's residual.
//
// On this part the FP64 pipe runs at 1/64 of the FP32 rate, so the mixed
// kernel computes the residual chain (displacement gradient, C, the
// material's S and J, -w F S G_a, the pressure terms) with pairs of floats
// x = h + l, |l| <= ulp(h) / 2, instead of doubles.  The building blocks are
// the error-free transformations TwoSum (Knuth) and TwoProd by FMA, and the
// compensated dot product Dot2 (Ogita, Rump, Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26, 2005); the pair operations follow the
// double-word algorithms analysed by Joldes, Muller and Popescu ("Tight and
// rigorous error bounds for basic building blocks of double-word
// arithmetic", ACM TOMS 44, 2017).  Each operation's error is a few units of
// 2^-48 relative to its operands, so the residual agrees with the FP64 path
// to ~1e-14 relative (the tests bound it at 1e-12).  The float exponent range
// applies: the mixed path needs |values| well inside 1e-30 .. 1e30.
// The intrinsics (__fadd_rn, __fmul_rn, __fmaf_rn) keep the compiler from
// contracting the transformations' separate roundings into FMAs.
struct dw {
  float h, l;
};

__device__ __forceinline__ dw two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ dw fast_two_sum(float a, float b) {  // |a| >= |b| (or a == 0)
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ dw two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ dw dw_neg(dw x) { return {-x.h, -x.l}; }
__device__ __forceinline__ dw dw_scale2(dw x, float p2) {  // p2 a power of two: exact
  return {x.h * p2, x.l * p2};
}

// x + y with error ~2^-47 (|x| + |y|)
__device__ __forceinline__ dw dw_add(dw x, dw y) {
  const dw s = two_sum(x.h, y.h);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(x.l, y.l)));
}

__device__ __forceinline__ dw dw_addf(dw x, float y) {
  const dw s = two_sum(x.h, y);
  return fast_two_sum(s.h, __fadd_rn(s.l, x.l));
}

__device__ __forceinline__ dw dw_mul(dw x, dw y) {
  const dw p = two_prod(x.h, y.h);
  return fast_two_sum(p.h, __fmaf_rn(x.h, y.l, __fmaf_rn(x.l, y.h, p.l)));
}

__device__ __forceinline__ dw dw_mulf(dw x, float y) {
  const dw p = two_prod(x.h, y);
  return fast_two_sum(p.h, __fmaf_rn(x.l, y, p.l));
}

// Dot2 accumulator: value s + c, c collects the rounding errors unnormalised
struct dacc {
  float s, c;
};

__device__ __forceinline__ void acc_prod(dacc& a, dw x, dw y) {
  const dw p = two_prod(x.h, y.h);
  const float e = __fmaf_rn(x.h, y.l, __fmaf_rn(x.l, y.h, p.l));
  const dw t = two_sum(a.s, p.h);
  a.s = t.h;
  a.c = __fadd_rn(a.c, __fadd_rn(t.l, e));
}

__device__ __forceinline__ void acc_add(dacc& a, dw x) {
  const dw t = two_sum(a.s, x.h);
  a.s = t.h;
  a.c = __fadd_rn(a.c, __fadd_rn(t.l, x.l));
}

__device__ __forceinline__ dw acc_val(dacc a) { return two_sum(a.s, a.c); }

__device__ __forceinline__ dw dw_of(float2 v) { return {v.x, v.y}; }

__device__ __forceinline__ dw dw_from_double(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - (double)h)};
}

// float -> double, exact, with integer operations: on this part the
// conversion instruction runs on the FP64 pipe, at its 1/64 rate, while a
// normal float widens by re-biasing the exponent (127 -> 1023) and shifting
// the mantissa, both on the integer pipe.  Zero is a select; subnormals,
// infinities and NaNs (none on the assembly's paths) take the conversion.
__device__ __forceinline__ double f2d(float f) {
  const uint32_t b = __float_as_uint(f);
  const uint32_t mag = b & 0x7FFFFFFFu;
  const uint32_t e = b & 0x7F800000u;
  if (mag != 0u && (e == 0u || e == 0x7F800000u)) return (double)f;
  const uint32_t sign = b & 0x80000000u;
  const uint32_t hi = mag ? (sign | ((mag >> 3) + (896u << 20))) : sign;
  const uint32_t lo = mag ? (b << 29) : 0u;
  return __hiloint2double((int)hi, (int)lo);
}

__device__ __forceinline__ double dw_to_double(dw x) { return f2d(x.h) + f2d(x.l); }

// sqrt(d): the float root refined by one Newton step on the pair
__device__ __forceinline__ dw dw_sqrt(dw d) {
  const float y = __fsqrt_rn(d.h);
  const dw yy = two_prod(y, y);
  const float r = __fadd_rn(__fsub_rn(__fsub_rn(d.h, yy.h), yy.l), d.l);  // d - y^2
  return fast_two_sum(y, __fdiv_rn(r, 2.0f * y));
}

// 1 / d: the float reciprocal refined by one Newton step
__device__ __forceinline__ dw dw_rcp(dw d) {
  const float y = __frcp_rn(d.h);
  const dw p = two_prod(d.h, y);
  const float r = __fsub_rn(__fsub_rn(1.0f, p.h), __fmaf_rn(d.l, y, p.l));  // 1 - d y
  return fast_two_sum(y, __fmul_rn(y, r));
}

// x^(-1/3): the float estimate refined by Newton steps on f(x) = x^-3 - J,
//   x' = x + x (1 - J x^3) / 3,   relative error e -> 2 e^2,
// two steps, since one leaves 2 (2^-23)^2 ~ 3e-14 from a 1-ulp estimate.
__device__ __forceinline__ dw dw_rcbrt(dw J) {
  const float x0 = rcbrtf(J.h);
  const dw t0 = dw_mul(J, dw_mulf(two_prod(x0, x0), x0));
  const float u0 = __fsub_rn(__fsub_rn(1.0f, t0.h), t0.l);  // 1 - J x^3 (t.h ~ 1: exact)
  const dw x1 = fast_two_sum(x0, __fmul_rn(x0, __fmul_rn(u0, 1.0f / 3.0f)));
  const dw t1 = dw_mul(J, dw_mul(dw_mul(x1, x1), x1));
  const float u1 = __fsub_rn(__fsub_rn(1.0f, t1.h), t1.l);
  return dw_add(x1, dw_mulf(x1, __fmul_rn(u1, 1.0f / 3.0f)));
}

// constants as pairs (the low parts folded at compile time)
#define NLA3D_DW_CONST(name, value) \
  constexpr float name##_h = (float)(value); \
  constexpr float name##_l = (float)((value) - (double)name##_h);
NLA3D_DW_CONST(kThird, 1.0 / 3.0)
NLA3D_DW_CONST(kTwoThirds, 2.0 / 3.0)
NLA3D_DW_CONST(kFourThirds, 4.0 / 3.0)
NLA3D_DW_CONST(kEightThirds, 8.0 / 3.0)
#undef NLA3D_DW_CONST

// a b - c d
__device__ __forceinline__ dw dw_diff_prod(dw a, dw b, dw c, dw d) {
  dacc t{0.0f, 0.0f};
  acc_prod(t, a, b);
  acc_prod(t, dw_neg(c), d);
  return acc_val(t);
}

// The material response of material<TT> with the state (S, J) in pairs and
// the tangent coefficients rounded to float (materials_hyperelastic.cpp:30-129,
// 135-204).
__device__ __forceinline__ void material_mixed(int mat_id, const float2* mcd, const dw C[6],
                                               dw p_state, dw p_cur, dw w, dw S[6], dw& Jout,
                                               float wD[21]) {
  const dw I1 = dw_add(dw_add(C[0], C[3]), C[5]);
  dacc t2{0.0f, 0.0f};
  acc_prod(t2, C[0], C[3]);
  acc_prod(t2, C[3], C[5]);
  acc_prod(t2, C[0], C[5]);
  acc_prod(t2, dw_neg(C[1]), C[1]);
  acc_prod(t2, dw_neg(C[4]), C[4]);
  acc_prod(t2, dw_neg(C[2]), C[2]);
  const dw I2 = acc_val(t2);
  // cofactors of the symmetric C: Ci = cof / det C
  dw cf[6];
  cf[0] = dw_diff_prod(C[3], C[5], C[4], C[4]);
  cf[1] = dw_diff_prod(C[2], C[4], C[1], C[5]);
  cf[2] = dw_diff_prod(C[1], C[4], C[2], C[3]);
  cf[3] = dw_diff_prod(C[0], C[5], C[2], C[2]);
  cf[4] = dw_diff_prod(C[1], C[2], C[0], C[4]);
  cf[5] = dw_diff_prod(C[0], C[3], C[1], C[1]);
  dacc td{0.0f, 0.0f};
  acc_prod(td, C[0], cf[0]);
  acc_prod(td, C[1], cf[1]);
  acc_prod(td, C[2], cf[2]);
  const dw detC = acc_val(td);
  const dw J = dw_sqrt(detC);
  const dw rc = dw_rcbrt(J);
  const dw pp = dw_mul(rc, rc);      // J^(-2/3)
  const dw pppp = dw_mul(pp, pp);    // J^(-4/3)
  const dw oo = dw_rcp(detC);        // 1 / J^2
  dw Ci[6];
#pragma unroll
  for (int i = 0; i < 6; i++) Ci[i] = dw_mul(oo, cf[i]);
  const dw t13 = dw_mul(I1, dw{kThird_h, kThird_l});
  const dw t23 = dw_mul(I2, dw{kTwoThirds_h, kTwoThirds_l});
  dw a1, a2{0.0f, 0.0f}, a11{0.0f, 0.0f};
  if (mat_id == 1) {
    a1 = dw_scale2(dw_of(mcd[0]), 0.5f);
  } else if (mat_id == 2) {
    const dw d = dw_addf(dw_mul(I1, pp), -3.0f);
    const dw m1 = dw_of(mcd[1]), m2 = dw_of(mcd[2]);
    dacc ta{0.0f, 0.0f};
    acc_add(ta, dw_of(mcd[0]));
    acc_prod(ta, dw_scale2(m1, 2.0f), d);
    acc_prod(ta, dw_mulf(m2, 3.0f), dw_mul(d, d));
    a1 = acc_val(ta);
    a2 = dw_of(mcd[3]);
    a11 = dw_add(dw_scale2(m1, 2.0f), dw_mul(dw_mulf(m2, 6.0f), d));
  } else {
    a1 = dw_of(mcd[0]);
    a2 = dw_of(mcd[1]);
  }
  const float I6[6] = {1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 1.0f};
  dw A[6], B[6];
#pragma unroll
  for (int i = 0; i < 6; i++) {
    A[i] = dw_addf(dw_neg(dw_mul(t13, Ci[i])), I6[i]);
    dacc tb{0.0f, 0.0f};
    acc_add(tb, dw_neg(C[i]));
    acc_prod(tb, dw_neg(t23), Ci[i]);
    if (I6[i] != 0.0f) acc_add(tb, I1);
    B[i] = acc_val(tb);
  }
  const dw ko1 = dw_scale2(dw_mul(a1, pp), 2.0f), ko2 = dw_scale2(dw_mul(a2, pppp), 2.0f);
  const dw pJs = dw_mul(p_state, J);
#pragma unroll
  for (int i = 0; i < 6; i++) {
    dacc ts{0.0f, 0.0f};
    acc_prod(ts, ko1, A[i]);
    acc_prod(ts, ko2, B[i]);
    acc_prod(ts, pJs, Ci[i]);
    S[i] = acc_val(ts);
  }
  Jout = J;
  // tangent coefficients (Dd before the reference's /2, times w), in float
  const dw k11 = dw_scale2(dw_mul(a11, pppp), 4.0f);
  const dw k1 = dw_mul(dw_mul(a1, pp), dw{kFourThirds_h, kFourThirds_l});
  const dw k2 = dw_mul(dw_mul(a2, pppp), dw{kEightThirds_h, kEightThirds_l});
  const dw pj = dw_mul(p_cur, J);
  dacc tc0{0.0f, 0.0f};
  acc_add(tc0, pj);
  acc_prod(tc0, dw_neg(k1), t13);
  acc_prod(tc0, dw_neg(k2), t23);
  const dw c0 = acc_val(tc0);
  dacc tst{0.0f, 0.0f};
  acc_add(tst, dw_scale2(pj, 2.0f));
  acc_prod(tst, dw_neg(k1), I1);
  acc_prod(tst, dw_neg(k2), I2);
  const float wf = w.h;
  const float sIIt = wf * acc_val(tst).h;
  const float sI = wf * 1.5f * k2.h;
  float At[6], Bt[6], Ct[6];
#pragma unroll
  for (int i = 0; i < 6; i++) {
    At[i] = A[i].h;
    Bt[i] = B[i].h;
    Ct[i] = Ci[i].h;
  }
  tangent_from_coefficients<float>(At, Bt, Ct, wf * k11.h, wf * k1.h, wf * k2.h, wf * c0.h, sIIt,
                                   sI, wD);
}

template <typename TT, int WPB>
__global__ void __launch_bounds__(WPB * 32)
    solid81_kernel(const Solid81Args a) {
  if (a.skip && *a.skip) return;
  constexpr bool kMixed = std::is_same<TT, float>::value;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // block header: the FP64 kernel's Kuu ownership words, the mixed kernel's
  // D -> assemble3 position table
  uint32_t* dec = reinterpret_cast<uint32_t*>(smem_raw);  // [kOwned64][32]
  // FP64 kernel: each owned entry's stage position, and the derived entries'
  // table (per-lane indices: shared memory, not the constant cache)
  uint16_t* opos = reinterpret_cast<uint16_t*>(dec + kOwned64 * 32);   // [kOwned64][32]
  uint16_t* dtab = opos + kOwned64 * 32;                               // [kKuuDerived][8]
  uint16_t* dpos = reinterpret_cast<uint16_t*>(smem_raw);  // [kDpos]
  constexpr size_t kHead = kMixed ? kDposBytes : kHead64Bytes;
  WarpSmem<TT>* sm = reinterpret_cast<WarpSmem<TT>*>(smem_raw + kHead) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;

  if constexpr (kMixed) {
    for (int v = threadIdx.x; v < kDpos; v += blockDim.x) dpos[v] = c_dpos[v];
  } else
  // Ownership of Kuu entries: lane owns x = lane + 32 m of the 4*231 owned
  // entries of its warp's element quad.  Decode once: smem offsets of
  // H[ik][.][slot a] and G[.][slot b].
  for (int v = threadIdx.x; v < kOwned64 * 32; v += blockDim.x) {
    const int m = v / 32, l = v % 32;
    const int x = l + 32 * m;
    // entries past the quad's 924 read slot 0 (in bounds) and are never written
    uint32_t word = 0u;
    uint16_t where = 0xFFFFu;
    if (x < kEPW * kKuuOwned) {
      const int q = x / kKuuOwned;
      const int t = c_kuu_owned[x - q * kKuuOwned];
      where = (uint16_t)(q * kKuuPerElem + t);
      const uchar4 en = c_kuu_entry[t];  // (a, i, b, k)
      // i <= k: h_a[ik] . G_b;  i > k: h_b[ki] . G_a (A symmetric)
      const bool up = en.y <= en.w;
      const uint32_t hb = up ? hblock(en.y, en.w) : hblock(en.w, en.y);
      const uint32_t ho = hb * kHStride + q * 8 + (up ? en.x : en.z);
      const uint32_t go = q * 8 + (up ? en.z : en.x);
      word = ho | (go << 16);
    }
    dec[m * 32 + l] = word;
    opos[m * 32 + l] = where;
  }
  if constexpr (!kMixed)
    for (int v = threadIdx.x; v < kKuuDerived * 8; v += blockDim.x) dtab[v] = c_kuu_derived[v];
  __syncthreads();

  const uint32_t E = a.n_elems;  // end of this launch's element range
  const uint64_t E8 = (uint64_t)(a.n_total ? a.n_total : E) * 8;
  const uint64_t n_quads = (E + kEPW - 1) / kEPW;
  const uint64_t warp_global = (uint64_t)blockIdx.x * WPB + (threadIdx.x >> 5);
  const uint64_t warp_stride = (uint64_t)gridDim.x * WPB;

  for (uint64_t quad = a.e_begin / kEPW + warp_global; quad < n_quads; quad += warp_stride) {
    const uint32_t e0 = (uint32_t)(quad * kEPW);
    const int q = lane >> 3;
    const int sub = lane & 7;  // Gauss point in phase 1, node in phase 2
    const uint32_t e = e0 + q;
    const bool valid = e < E;
    const uint32_t ec = valid ? e : E - 1;

    // ---------------- phase 1: lane = (element q, Gauss point g) ----------------
    double Fp_part = 0.0, Kpp_part = 0.0;  // FP64 in both kernels
    {
      const int g = sub;
      const uint64_t tg = (uint64_t)ec * 8 + g;
      TT Fm[9], wS[6], wD[21];
      bool bad;
      if constexpr (kMixed) {
        // the residual chain in float pairs, the tangent inputs rounded to float
        const dw w = dw_of(__ldg(a.wdf + tg));
        const dw pc = dw_from_double(a.U_cur[a.p_eq[ec] - 1]);
        dw O[9];
        dw C[6];
        dw ps{0.0f, 0.0f};
        if (a.have_state) {
          // O = sum_n (u_n - u_0) G_n (the shape gradients sum to zero): the
          // displacements relative to the element's node 0 are formed in FP64,
          // so the pairs carry the small differences, not |u| (which can be
          // ~1/h times larger, and would cost that factor in accuracy).
          // Lane (q, g) forms node g's difference; the others read it by shuffle.
          const uint32_t* cn = a.conn + (uint64_t)ec * 8;
          const uint4 eq0 = __ldg(reinterpret_cast<const uint4*>(a.node_eq3) + (__ldg(cn) - 1));
          const uint4 eqg = __ldg(reinterpret_cast<const uint4*>(a.node_eq3) + (__ldg(cn + g) - 1));
          const dw dx = dw_from_double(a.U_state[eqg.x - 1] - a.U_state[eq0.x - 1]);
          const dw dy = dw_from_double(a.U_state[eqg.y - 1] - a.U_state[eq0.y - 1]);
          const dw dz = dw_from_double(a.U_state[eqg.z - 1] - a.U_state[eq0.z - 1]);
          dw G[24];
#pragma unroll
          for (int c = 0; c < 24; c++) G[c] = dw_of(__ldg(a.Gdf + c * E8 + tg));
          dacc Oa[9];
#pragma unroll
          for (int c = 0; c < 9; c++) Oa[c] = dacc{0.0f, 0.0f};
          const int base = lane & ~7;
#pragma unroll
          for (int n = 1; n < 8; n++) {
            const dw ux{__shfl_sync(0xFFFFFFFFu, dx.h, base + n), __shfl_sync(0xFFFFFFFFu, dx.l, base + n)};
            const dw uy{__shfl_sync(0xFFFFFFFFu, dy.h, base + n), __shfl_sync(0xFFFFFFFFu, dy.l, base + n)};
            const dw uz{__shfl_sync(0xFFFFFFFFu, dz.h, base + n), __shfl_sync(0xFFFFFFFFu, dz.l, base + n)};
#pragma unroll
            for (int j = 0; j < 3; j++) {
              acc_prod(Oa[0 + j], ux, G[3 * n + j]);
              acc_prod(Oa[3 + j], uy, G[3 * n + j]);
              acc_prod(Oa[6 + j], uz, G[3 * n + j]);
            }
          }
#pragma unroll
          for (int c = 0; c < 9; c++) O[c] = acc_val(Oa[c]);
          ps = dw_from_double(a.U_state[a.p_eq[ec] - 1]);
          // C = F^T F = I + O + O^T + O^T O (SOLID81.cpp:105-110)
          const int dg[3] = {0, 4, 8};
          const int cj[6] = {0, 0, 0, 1, 1, 2}, cl[6] = {0, 1, 2, 1, 2, 2};
#pragma unroll
          for (int v = 0; v < 6; v++) {
            const int J = cj[v], L = cl[v];
            dacc t{J == L ? 1.0f : 0.0f, 0.0f};
            if (J == L) {
              acc_add(t, dw_scale2(O[dg[J]], 2.0f));
            } else {
              acc_add(t, O[3 * J + L]);
              acc_add(t, O[3 * L + J]);
            }
#pragma unroll
            for (int i = 0; i < 3; i++) acc_prod(t, O[3 * i + J], O[3 * i + L]);
            C[v] = acc_val(t);
          }
        } else {
#pragma unroll
          for (int c = 0; c < 9; c++) O[c] = dw{0.0f, 0.0f};
          C[0] = C[3] = C[5] = dw{1.0f, 0.0f};
          C[1] = C[2] = C[4] = dw{0.0f, 0.0f};
        }
        int mat_id = a.mat_id;
        const float2* mcd = a.mcd;
        if (a.elem_mesh) {
          const uint32_t mi = __ldg(a.elem_mesh + ec);
          mat_id = (int)a.mesh_mat[8 * (uint64_t)mi];
          mcd = a.mesh_mat_df + 8 * (uint64_t)mi + 1;
        }
        dw S[6], J;
        material_mixed(mat_id, mcd, C, ps, pc, w, S, J, wD);
        if (!a.have_state) {
#pragma unroll
          for (int i = 0; i < 6; i++) S[i] = dw{0.0f, 0.0f};
        }
        dw F[9];
#pragma unroll
        for (int c = 0; c < 9; c++) F[c] = (c == 0 || c == 4 || c == 8) ? dw_addf(O[c], 1.0f) : O[c];
        const int sv[9] = {0, 1, 2, 1, 3, 4, 2, 4, 5};
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int k = 0; k < 3; k++) {
            dacc t{0.0f, 0.0f};
#pragma unroll
            for (int J2 = 0; J2 < 3; J2++) acc_prod(t, F[3 * i + J2], S[sv[3 * J2 + k]]);
            const dw wp = dw_mul(w, acc_val(t));
            // slot g * 4 + q: the four elements' pairs of one Gauss point
            // fall in different bank pairs when phase 2 reads them
            sm->wP[3 * i + k][g * 4 + q] = make_float2(-wp.h, -wp.l);
          }
#pragma unroll
        for (int c = 0; c < 9; c++) Fm[c] = F[c].h;
#pragma unroll
        for (int c = 0; c < 6; c++) wS[c] = w.h * S[c].h;
        // The volumetric terms in FP64: F (the pair O widened exactly, plus
        // I), cof F, J = det F, and from them Fp = -(J - 1 - p / K) w,
        // Kpp = -w / K (SOLID81.cpp:78-79) and w cof F = w J F^-T, whose
        // products with G_a are K_up (D_p = J C^-1, materials_hyperelastic.cpp:127).
        double Fd[9];
#pragma unroll
        for (int c = 0; c < 9; c++) {
          const double o = dw_to_double(O[c]);
          Fd[c] = (c == 0 || c == 4 || c == 8) ? 1.0 + o : o;
        }
        const double cofd[9] = {Fd[4] * Fd[8] - Fd[5] * Fd[7], Fd[5] * Fd[6] - Fd[3] * Fd[8],
                                Fd[3] * Fd[7] - Fd[4] * Fd[6], Fd[2] * Fd[7] - Fd[1] * Fd[8],
                                Fd[0] * Fd[8] - Fd[2] * Fd[6], Fd[1] * Fd[6] - Fd[0] * Fd[7],
                                Fd[1] * Fd[5] - Fd[2] * Fd[4], Fd[2] * Fd[3] - Fd[0] * Fd[5],
                                Fd[0] * Fd[4] - Fd[1] * Fd[3]};
        const double wd = a.wdet[tg];
#pragma unroll
        for (int c = 0; c < 9; c++) sm->wCof[c][g * 4 + q] = wd * cofd[c];
        {
          const float cf[9] = {Fm[4] * Fm[8] - Fm[5] * Fm[7], Fm[5] * Fm[6] - Fm[3] * Fm[8],
                               Fm[3] * Fm[7] - Fm[4] * Fm[6], Fm[2] * Fm[7] - Fm[1] * Fm[8],
                               Fm[0] * Fm[8] - Fm[2] * Fm[6], Fm[1] * Fm[6] - Fm[0] * Fm[7],
                               Fm[1] * Fm[5] - Fm[2] * Fm[4], Fm[2] * Fm[3] - Fm[0] * Fm[5],
                               Fm[0] * Fm[4] - Fm[1] * Fm[3]};
#pragma unroll
          for (int c = 0; c < 9; c++) sm->wCofF[c][g * 4 + q] = w.h * cf[c];
        }
        const double Jd = Fd[0] * cofd[0] + Fd[1] * cofd[1] + Fd[2] * cofd[2];
        const double inv_kbd =
            a.elem_mesh ? a.mesh_mat[8 * (uint64_t)__ldg(a.elem_mesh + ec) + 7] : a.inv_kb;
        const double pcd = a.U_cur[a.p_eq[ec] - 1];
        Fp_part = -(Jd - 1 - pcd * inv_kbd) * wd;
        Kpp_part = -inv_kbd * wd;
        bad = valid && !(Jd > 0.0 && isfinite(Jd) && J.h > 0.0f && isfinite(J.h) && wd > 0.0);
      } else {
        const double w = a.wdet[tg];
        const double pc = a.U_cur[a.p_eq[ec] - 1];
        double O[9];
        double C[6];
        double ps = 0.0;
        if (a.have_state) {
          double G[24];
#pragma unroll
          for (int c = 0; c < 24; c++) G[c] = __ldg(a.Gt + c * E8 + tg);
#pragma unroll
          for (int c = 0; c < 9; c++) O[c] = 0.0;
#pragma unroll
          for (int n = 0; n < 8; n++) {
            const uint32_t nid = __ldg(a.conn + (uint64_t)ec * 8 + n);
            const uint4 eq = __ldg(reinterpret_cast<const uint4*>(a.node_eq3) + (nid - 1));
            const double ux = a.U_state[eq.x - 1], uy = a.U_state[eq.y - 1],
                         uz = a.U_state[eq.z - 1];
#pragma unroll
            for (int j = 0; j < 3; j++) {
              O[0 + j] = fma(ux, G[3 * n + j], O[0 + j]);
              O[3 + j] = fma(uy, G[3 * n + j], O[3 + j]);
              O[6 + j] = fma(uz, G[3 * n + j], O[6 + j]);
            }
          }
          ps = a.U_state[a.p_eq[ec] - 1];
          // C = F^T F from O (SOLID81.cpp:105-110)
          C[0] = 1.0 + 2 * O[0] + O[0] * O[0] + O[3] * O[3] + O[6] * O[6];
          C[3] = 1.0 + 2 * O[4] + O[1] * O[1] + O[4] * O[4] + O[7] * O[7];
          C[5] = 1.0 + 2 * O[8] + O[2] * O[2] + O[5] * O[5] + O[8] * O[8];
          C[1] = O[1] + O[3] + O[0] * O[1] + O[3] * O[4] + O[6] * O[7];
          C[4] = O[5] + O[7] + O[1] * O[2] + O[4] * O[5] + O[7] * O[8];
          C[2] = O[2] + O[6] + O[0] * O[2] + O[3] * O[5] + O[6] * O[8];
        } else {
          // state right after Element::pre(): C = I, S = 0, O = 0 (SOLID81.cpp:17-19)
#pragma unroll
          for (int c = 0; c < 9; c++) O[c] = 0.0;
          C[0] = C[3] = C[5] = 1.0;
          C[1] = C[2] = C[4] = 0.0;
        }
        int mat_id = a.mat_id;
        const double* mc = a.mc;
        double kbulk = a.kbulk;
        if (a.elem_mesh) {
          const double* mm = a.mesh_mat + 8 * (uint64_t)__ldg(a.elem_mesh + ec);
          mat_id = (int)mm[0];
          mc = mm + 1;
          kbulk = mm[6];
        }
        const double inv_kb = 1.0 / kbulk;
        MatOut<TT> mo;
        material<TT>(mat_id, mc, C, ps, pc, w, mo, wD);
        if (!a.have_state) {
#pragma unroll
          for (int i = 0; i < 6; i++) mo.S[i] = 0.0;
        }
        const double J = mo.J;
        const double F[9] = {1.0 + O[0], O[1], O[2], O[3], 1.0 + O[4], O[5], O[6], O[7], 1.0 + O[8]};
        const double S3[9] = {mo.S[0], mo.S[1], mo.S[2], mo.S[1], mo.S[3], mo.S[4],
                              mo.S[2], mo.S[4], mo.S[5]};
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int k = 0; k < 3; k++) {
            const double fs = F[3 * i + 0] * S3[0 + k] + F[3 * i + 1] * S3[3 + k] +
                              F[3 * i + 2] * S3[6 + k];
            sm->wP[3 * i + k][lane] = -w * fs;
          }
        const double cof[9] = {F[4] * F[8] - F[5] * F[7], F[5] * F[6] - F[3] * F[8],
                               F[3] * F[7] - F[4] * F[6], F[2] * F[7] - F[1] * F[8],
                               F[0] * F[8] - F[2] * F[6], F[1] * F[6] - F[0] * F[7],
                               F[1] * F[5] - F[2] * F[4], F[2] * F[3] - F[0] * F[5],
                               F[0] * F[4] - F[1] * F[3]};
#pragma unroll
        for (int c = 0; c < 9; c++) sm->wCof[c][lane] = w * cof[c];
#pragma unroll
        for (int c = 0; c < 9; c++) Fm[c] = (TT)F[c];
#pragma unroll
        for (int c = 0; c < 6; c++) wS[c] = (TT)(w * mo.S[c]);
        Fp_part = -(J - 1 - pc * inv_kb) * w;
        Kpp_part = -inv_kb * w;
        // J = sqrt(det C) cannot see an inverted element; det F can
        const double detF = F[0] * cof[0] + F[1] * cof[1] + F[2] * cof[2];
        bad = valid && !(J > 0.0 && isfinite(J) && detF > 0.0 && w > 0.0);
      }
      // A[iL][kN] = sum_J F_iJ (sum_M wD[(JL)][(MN)] F_kM) + delta_ik w S_LN,
      // one row (i, L) at a time
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int L = 0; L < 3; L++) {
          TT T6[6];
#pragma unroll
          for (int t = 0; t < 6; t++)
            T6[t] = Fm[3 * i + 0] * wD[sym6u(voigt(0, L), t)] +
                    Fm[3 * i + 1] * wD[sym6u(voigt(1, L), t)] +
                    Fm[3 * i + 2] * wD[sym6u(voigt(2, L), t)];
#pragma unroll
          for (int k = 0; k < 3; k++)
#pragma unroll
            for (int N = 0; N < 3; N++) {
              if (3 * k + N < 3 * i + L) continue;
              TT v = T6[voigt(0, N)] * Fm[3 * k + 0] + T6[voigt(1, N)] * Fm[3 * k + 1] +
                     T6[voigt(2, N)] * Fm[3 * k + 2];
              if (i == k) v += wS[voigt(L, N)];
              sm->A[sym9(3 * i + L, 3 * k + N)][lane] = v;
            }
        }
      const unsigned ballot = __ballot_sync(0xFFFFFFFFu, bad);
      if (sub == 0 && ((ballot >> (q * 8)) & 0xFFu)) flag_element(a.status, e + 1);
    }
#pragma unroll
    for (int off = 1; off < 8; off <<= 1) {
      Fp_part += __shfl_xor_sync(0xFFFFFFFFu, Fp_part, off);
      Kpp_part += __shfl_xor_sync(0xFFFFFFFFu, Kpp_part, off);
    }
    __syncwarp();

    // destination of contribution idx: slot-ordered (kpos) or element-ordered
    auto kdst = [&](uint64_t idx) -> uint64_t { return a.kpos ? (uint64_t)__ldg(a.kpos + idx) : idx; };
    auto fdst = [&](uint64_t idx) -> uint64_t { return a.fpos ? (uint64_t)__ldg(a.fpos + idx) : idx; };

    if constexpr (kMixed) {
      // Residual and pressure coupling, lane = (element q, node a), before the
      // Gauss point loop reuses the scratch that holds -w F S and w cof F:
      //   F_u(a, i) = sum_g sum_L (-w F S)_g[iL] G_g[aL]   (float pairs),
      //   K_up(a, i) = sum_g sum_L (w cof F)_g[iL] G_g[aL]  (FP64),
      // G = G_hi + G_lo its pair.  The K_up products with G_hi are FP64 FMAs
      // (two accumulators, even and odd Gauss points, to halve the dependent
      // chain); the products with G_lo, 2^-24 of the total, are summed in
      // FP32 (their error, 2^-48 of the total, is that of the pair itself)
      // and added in FP64 at the end.  The pair arithmetic of F_u keeps the
      // FP32 pipes busy while the FP64 FMAs drain.  Kpp and Fp are written
      // here too.
      double Kupd[2][3] = {{0.0, 0.0, 0.0}, {0.0, 0.0, 0.0}};
      float Kupl[3] = {0.0f, 0.0f, 0.0f};
      dacc Fua[3] = {{0.0f, 0.0f}, {0.0f, 0.0f}, {0.0f, 0.0f}};
#pragma unroll 2
      for (int g = 0; g < 8; g++) {
        const uint64_t tg = (uint64_t)ec * 8 + g;
        const float2 p0 = __ldg(a.Gdf + (3 * sub + 0) * E8 + tg);
        const float2 p1 = __ldg(a.Gdf + (3 * sub + 1) * E8 + tg);
        const float2 p2 = __ldg(a.Gdf + (3 * sub + 2) * E8 + tg);
        const double G0 = f2d(p0.x), G1 = f2d(p1.x), G2 = f2d(p2.x);
        const int sp = g * 4 + q;
#pragma unroll
        for (int i = 0; i < 3; i++) {
          double& kd = Kupd[g & 1][i];
          kd = fma(sm->wCof[3 * i + 0][sp], G0, kd);
          kd = fma(sm->wCof[3 * i + 1][sp], G1, kd);
          kd = fma(sm->wCof[3 * i + 2][sp], G2, kd);
          Kupl[i] += sm->wCofF[3 * i + 0][sp] * p0.y + sm->wCofF[3 * i + 1][sp] * p1.y +
                     sm->wCofF[3 * i + 2][sp] * p2.y;
          acc_prod(Fua[i], dw_of(sm->wP[3 * i + 0][sp]), dw_of(p0));
          acc_prod(Fua[i], dw_of(sm->wP[3 * i + 1][sp]), dw_of(p1));
          acc_prod(Fua[i], dw_of(sm->wP[3 * i + 2][sp]), dw_of(p2));
        }
      }
      if (valid) {
        const uint64_t kb = (uint64_t)e * kSolidKc, fb = (uint64_t)e * kSolidFc;
#pragma unroll
        for (int i = 0; i < 3; i++) {
          a.contribK[kdst(kb + 300 + 3 * sub + i)] = (Kupd[0][i] + Kupd[1][i]) + f2d(Kupl[i]);
          a.contribF[fdst(fb + 3 * sub + i)] = dw_to_double(acc_val(Fua[i]));
        }
        if (sub == 0) {
          a.contribK[kdst(kb + 324)] = Kpp_part;
          a.contribF[fdst(fb + 24)] = Fp_part;
        }
      }
      __syncwarp();
    }

    // ---------------- phases 2 + 3 per Gauss point ----------------
    if constexpr (kMixed) {
      // Lane (q, a) keeps h_a[ik] (i <= k, its own node) in registers and
      // accumulates D[(ik), a, b] = sum_g h_a[ik] . G_b for all 8 nodes b:
      // 48 sums of 3 FMA per Gauss point from 3 shared loads per node b.
      // The 48 cover the element's 300 Kuu entries (the 84 D[(ii), a, b],
      // a > b, repeat D[(ii), b, a] and are not written).
      float acc[6][8];
#pragma unroll
      for (int c = 0; c < 6; c++)
#pragma unroll
        for (int b = 0; b < 8; b++) acc[c][b] = 0.0f;
      for (int g = 0; g < 8; g++) {
        const int s1 = q * 8 + g;
        const uint64_t tg = (uint64_t)ec * 8 + g;
        // phase 2: the tangent uses the high parts of G
        const float g0 = __ldg(a.Gdf + (3 * sub + 0) * E8 + tg).x;
        const float g1 = __ldg(a.Gdf + (3 * sub + 1) * E8 + tg).x;
        const float g2 = __ldg(a.Gdf + (3 * sub + 2) * E8 + tg).x;
        float h[6][3];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int k = i; k < 3; k++)
#pragma unroll
            for (int N = 0; N < 3; N++)
              h[hblock(i, k)][N] = g0 * sm->A[sym9(3 * i + 0, 3 * k + N)][s1] +
                                   g1 * sm->A[sym9(3 * i + 1, 3 * k + N)][s1] +
                                   g2 * sm->A[sym9(3 * i + 2, 3 * k + N)][s1];
        sm->G[0][lane] = g0;
        sm->G[1][lane] = g1;
        sm->G[2][lane] = g2;
        __syncwarp();
        // phase 3
#pragma unroll
        for (int b = 0; b < 8; b++) {
          const float b0 = sm->G[0][q * 8 + b], b1 = sm->G[1][q * 8 + b],
                      b2 = sm->G[2][q * 8 + b];
#pragma unroll
          for (int c = 0; c < 6; c++) {
            float v = acc[c][b];
            v = fmaf(h[c][0], b0, v);
            v = fmaf(h[c][1], b1, v);
            v = fmaf(h[c][2], b2, v);
            acc[c][b] = v;
          }
        }
        __syncwarp();
      }
      // stage the quad's 4 x 300 entries in assemble3 order, then write them
      // coalesced (the stage shares its bytes with -w F S / w cof F, dead now)
#pragma unroll
      for (int c = 0; c < 6; c++)
#pragma unroll
        for (int b = 0; b < 8; b++) {
          const uint32_t pos = dpos[(sub * 6 + c) * 8 + b];
          if (pos != 0xFFFFu) sm->stage[q * kKuuPerElem + pos] = acc[c][b];
        }
      __syncwarp();
#pragma unroll 4
      for (int m = 0; m < kOwned; m++) {
        const int x = lane + 32 * m;
        if (x < kEPW * kKuuPerElem) {
          const int qq = x / kKuuPerElem, t = x - qq * kKuuPerElem;
          const uint32_t ee = e0 + qq;
          if (ee < E) a.contribK[kdst((uint64_t)ee * kSolidKc + t)] = f2d(sm->stage[x]);
        }
      }
      __syncwarp();
    } else {
    TT acc[kOwned64];
#pragma unroll
    for (int m = 0; m < kOwned64; m++) acc[m] = (TT)0;
    double Fu[3] = {0.0, 0.0, 0.0};   // FP64 kernel (the mixed one wrote F_u and
    double Kup[3] = {0.0, 0.0, 0.0};  // K_up above)
    const int node = sub;
    for (int g = 0; g < 8; g++) {
      const int s1 = q * 8 + g;
      {
        // phase 2: lane = (element q, node a)
        const uint64_t tg = (uint64_t)ec * 8 + g;
        TT gg[3];
        if constexpr (kMixed) {
          // the tangent uses the high parts
          gg[0] = __ldg(a.Gdf + (3 * node + 0) * E8 + tg).x;
          gg[1] = __ldg(a.Gdf + (3 * node + 1) * E8 + tg).x;
          gg[2] = __ldg(a.Gdf + (3 * node + 2) * E8 + tg).x;
        } else {
          const double G0 = __ldg(a.Gt + (3 * node + 0) * E8 + tg);
          const double G1 = __ldg(a.Gt + (3 * node + 1) * E8 + tg);
          const double G2 = __ldg(a.Gt + (3 * node + 2) * E8 + tg);
          // residual and pressure coupling in FP64, one FMA chain per entry
          // (three FMAs per Gauss point instead of a product, two FMAs and an add)
#pragma unroll
          for (int i = 0; i < 3; i++) {
            Fu[i] = fma(sm->wP[3 * i + 0][s1], G0, Fu[i]);
            Fu[i] = fma(sm->wP[3 * i + 1][s1], G1, Fu[i]);
            Fu[i] = fma(sm->wP[3 * i + 2][s1], G2, Fu[i]);
            Kup[i] = fma(sm->wCof[3 * i + 0][s1], G0, Kup[i]);
            Kup[i] = fma(sm->wCof[3 * i + 1][s1], G1, Kup[i]);
            Kup[i] = fma(sm->wCof[3 * i + 2][s1], G2, Kup[i]);
          }
          gg[0] = (TT)G0;
          gg[1] = (TT)G1;
          gg[2] = (TT)G2;
        }
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int k = i; k < 3; k++)
#pragma unroll
            for (int N = 0; N < 3; N++)
              sm->H[hblock(i, k) * kHStride + 32 * N + lane] =
                  gg[0] * sm->A[sym9(3 * i + 0, 3 * k + N)][s1] +
                  gg[1] * sm->A[sym9(3 * i + 1, 3 * k + N)][s1] +
                  gg[2] * sm->A[sym9(3 * i + 2, 3 * k + N)][s1];
#pragma unroll
        for (int c = 0; c < 3; c++) sm->G[c][lane] = gg[c];
      }
      __syncwarp();
      {
        // phase 3: owned Kuu entries, K(a,i; b,k) += h_a[ik] . G_b
        const TT* Hf = sm->H;
        const TT* Gf = &sm->G[0][0];
#pragma unroll
        for (int m = 0; m < kOwned64; m++) {
          const uint32_t word = dec[m * 32 + lane];
          const uint32_t ho = word & 0xFFFFu, go = word >> 16;
          TT v = acc[m];
          v += Hf[ho] * Gf[go];
          v += Hf[ho + 32] * Gf[go + 32];
          v += Hf[ho + 64] * Gf[go + 64];
          acc[m] = v;
        }
      }
      __syncwarp();
    }

    // ---------------- write the element contributions ----------------
    // the owned entries into the quad's stage (assemble3 order; A's scratch,
    // dead after the Gauss-point loop), node 7's column from them, node 7's
    // block from that column, then all 4 x 300 written coalesced
    TT* stage = &sm->A[0][0];
#pragma unroll
    for (int m = 0; m < kOwned64; m++) {
      const uint16_t where = opos[m * 32 + lane];
      if (where != 0xFFFFu) stage[where] = acc[m];
    }
    __syncwarp();
    for (int dx = lane; dx < kEPW * kKuuColumn; dx += 32) {
      const int qq = dx / kKuuColumn, j = dx - qq * kKuuColumn;
      const TT* st = stage + qq * kKuuPerElem;
      const uint16_t* dj = dtab + j * 8;
      TT v = st[dj[1]];
#pragma unroll
      for (int c = 2; c < 8; c++) v += st[dj[c]];
      stage[qq * kKuuPerElem + dj[0]] = -v;
    }
    __syncwarp();
    if (lane < kEPW * kKuuCorner) {
      const int qq = lane / kKuuCorner, j = kKuuColumn + lane - qq * kKuuCorner;
      const TT* st = stage + qq * kKuuPerElem;
      const uint16_t* dj = dtab + j * 8;
      TT v = st[dj[1]];
#pragma unroll
      for (int c = 2; c < 8; c++) v += st[dj[c]];
      stage[qq * kKuuPerElem + dj[0]] = -v;
    }
    __syncwarp();
#pragma unroll 4
    for (int m = 0; m < kOwned; m++) {
      const int x = lane + 32 * m;
      if (x < kEPW * kKuuPerElem) {
        const int qq = x / kKuuPerElem, t = x - qq * kKuuPerElem;
        const uint32_t ee = e0 + qq;
        if (ee < E) a.contribK[kdst((uint64_t)ee * kSolidKc + t)] = stage[x];
      }
    }
    if (valid) {
      const uint64_t kb = (uint64_t)e * kSolidKc, fb = (uint64_t)e * kSolidFc;
#pragma unroll
      for (int i = 0; i < 3; i++) {
        a.contribK[kdst(kb + 300 + 3 * node + i)] = Kup[i];
        a.contribF[fdst(fb + 3 * node + i)] = Fu[i];
      }
      if (node == 0) {
        a.contribK[kdst(kb + 324)] = Kpp_part;
        a.contribF[fdst(fb + 24)] = Fp_part;
      }
    }
    __syncwarp();
    }  // FP64 kernel
  }
}

__global__ void solid81_jacobian_kernel(const JacobianArgs a) {
  if (a.skip && *a.skip) return;
  const uint64_t E8 = (uint64_t)a.n_elems * 8;
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= E8) return;
  const uint32_t e = (uint32_t)(t >> 3);
  const int g = (int)(t & 7);
  // Gauss point of ElementIsoParamHEXAHEDRON, order 2 (isoparametric.h:126-136)
  const double r = (g & 1) ? kGaussA : -kGaussA;
  const double s = (g & 2) ? kGaussA : -kGaussA;
  const double u = (g & 4) ? kGaussA : -kGaussA;
  // formFuncDeriv (isoparametric.cpp:211-221)
  const double dN[24] = {
      -0.125 * (1.0 - s) * (1.0 - u), -0.125 * (1.0 - r) * (1.0 - u), -0.125 * (1.0 - r) * (1.0 - s),
      +0.125 * (1.0 - s) * (1.0 - u), -0.125 * (1.0 + r) * (1.0 - u), -0.125 * (1.0 + r) * (1.0 - s),
      +0.125 * (1.0 + s) * (1.0 - u), +0.125 * (1.0 + r) * (1.0 - u), -0.125 * (1.0 + r) * (1.0 + s),
      -0.125 * (1.0 + s) * (1.0 - u), +0.125 * (1.0 - r) * (1.0 - u), -0.125 * (1.0 - r) * (1.0 + s),
      -0.125 * (1.0 - s) * (1.0 + u), -0.125 * (1.0 - r) * (1.0 + u), +0.125 * (1.0 - r) * (1.0 - s),
      +0.125 * (1.0 - s) * (1.0 + u), -0.125 * (1.0 + r) * (1.0 + u), +0.125 * (1.0 + r) * (1.0 - s),
      +0.125 * (1.0 + s) * (1.0 + u), +0.125 * (1.0 + r) * (1.0 + u), +0.125 * (1.0 + r) * (1.0 + s),
      -0.125 * (1.0 + s) * (1.0 + u), +0.125 * (1.0 - r) * (1.0 + u), +0.125 * (1.0 - r) * (1.0 + s)};
  double J[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int n = 0; n < 8; n++) {
    const uint32_t nid = a.conn[(uint64_t)e * 8 + n];
    const double* X = a.xyz + (uint64_t)(nid - 1) * 3;
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) J[3 * i + j] += dN[3 * n + i] * X[j];
  }
  // Mat<3,3>::det / inv (Mat.cpp:23-46)
  const double det = J[0] * (J[4] * J[8] - J[5] * J[7]) - J[1] * (J[3] * J[8] - J[5] * J[6]) +
                     J[2] * (J[3] * J[7] - J[4] * J[6]);
  const double sc = 1.0 / det;
  const double Ji[9] = {(J[4] * J[8] - J[5] * J[7]) * sc, (J[2] * J[7] - J[1] * J[8]) * sc,
                        (J[1] * J[5] - J[2] * J[4]) * sc, (J[6] * J[5] - J[3] * J[8]) * sc,
                        (J[0] * J[8] - J[2] * J[6]) * sc, (J[3] * J[2] - J[0] * J[5]) * sc,
                        (J[3] * J[7] - J[4] * J[6]) * sc, (J[1] * J[6] - J[0] * J[7]) * sc,
                        (J[0] * J[4] - J[1] * J[3]) * sc};
  for (int n = 0; n < 8; n++)
    for (int i = 0; i < 3; i++) {
      double v = 0.0;
      for (int j = 0; j < 3; j++) v += Ji[3 * i + j] * dN[3 * n + j];
      if (a.Gt) a.Gt[(uint64_t)(3 * n + i) * E8 + t] = v;
      if (a.Gdf) {
        const dw p = dw_from_double(v);
        a.Gdf[(uint64_t)(3 * n + i) * E8 + t] = make_float2(p.h, p.l);
      }
    }
  a.wdet[t] = 1.0 * det;
  if (a.wdf) {
    const dw p = dw_from_double(1.0 * det);
    a.wdf[t] = make_float2(p.h, p.l);
  }
  // isoparametric.cpp:177 logs det < 1e-20; here it is an element status
  if (!(det >= 1.0e-20) && g == 0) flag_element(a.status, e + 1);
}

// K[s] = sum of its contributions in ascending contribution order (the
// reference's element-ascending accumulation order), starting from 0.
//
// The sums are FP64 adds, and on this part the FP64 pipe is the scarce unit:
// a warp pays for an add whenever any of its lanes needs one.  Slots have
// 1..8 contributions (a hexahedral mesh: 8 on a node's own diagonal, 4/2/1
// off it, 1 for every pressure coupling), so a warp of consecutive slots pays
// for 8 adds where its slots need ~2.2 on average.  Each block therefore
// first sorts its slots by contribution count (a counting sort in shared
// memory; which thread sums a slot does not change the slot's sum), so the
// warps see nearly uniform counts and stop adding at their own maximum.
// Up to kBatch loads of a slot are issued before the first add; the adds keep
// the ascending order, and 0 + c1 is taken as c1 with -0 turned into +0, so
// the result is bitwise the plain sequential loop's.
constexpr int kBatch = 8;
constexpr int kCountClasses = kBatch + 2;  // counts 0..kBatch, and more than kBatch
constexpr int kMaxGatherBlock = 1024;

__device__ __forceinline__ double plus_zero_sum(double x) {
  // 0.0 + x without an FP64 add: x, except -0.0 -> +0.0
  const long long b = __double_as_longlong(x);
  return __longlong_as_double(b == (long long)0x8000000000000000ull ? 0ll : b);
}

template <bool kIds>
__global__ void __launch_bounds__(kMaxGatherBlock)
    gather_sorted_kernel(const uint64_t s_begin, const uint64_t n_slots,
                         const uint32_t* __restrict__ ptr, const uint32_t* __restrict__ ids,
                         const double* __restrict__ contrib, double* __restrict__ out,
                         const uint32_t* __restrict__ skip) {
  if (skip && *skip) return;  // the same word for every thread: a uniform exit
  __shared__ uint32_t s_beg[kMaxGatherBlock];
  __shared__ uint32_t s_end[kMaxGatherBlock];
  __shared__ uint16_t s_slot[kMaxGatherBlock];
  __shared__ uint32_t s_wcnt[kMaxGatherBlock / 32][kCountClasses];
  __shared__ uint32_t s_total[kCountClasses];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int n_warps = blockDim.x >> 5;
  const uint64_t base = s_begin + (uint64_t)blockIdx.x * blockDim.x;
  const uint64_t s = base + tid;
  uint32_t b = 0, e = 0;
  if (s < n_slots) {
    b = __ldg(ptr + s);
    e = __ldg(ptr + s + 1);
  }
  s_beg[tid] = b;
  s_end[tid] = e;
  const uint32_t n = e - b;
  const int cls = n > (uint32_t)kBatch ? kBatch + 1 : (int)n;
  // rank within (warp, class), and per-warp class counts
  if (lane < kCountClasses) s_wcnt[warp][lane] = 0;
  __syncwarp();
  const unsigned same = __match_any_sync(0xFFFFFFFFu, cls);
  const uint32_t rank = __popc(same & ((1u << lane) - 1u));
  if (rank == 0) s_wcnt[warp][cls] = __popc(same);
  __syncthreads();
  // exclusive prefix over warps, per class (one thread per class)
  if (tid < kCountClasses) {
    uint32_t run = 0;
    for (int w = 0; w < n_warps; w++) {
      const uint32_t t = s_wcnt[w][tid];
      s_wcnt[w][tid] = run;
      run += t;
    }
    s_total[tid] = run;
  }
  __syncthreads();
  uint32_t pos = s_wcnt[warp][cls] + rank;
  for (int c = 0; c < cls; c++) pos += s_total[c];
  s_slot[pos] = (uint16_t)tid;
  __syncthreads();

  const int lt = s_slot[tid];
  const uint64_t slot = base + lt;
  const uint32_t sb = s_beg[lt], se = s_end[lt];
  const uint32_t sn = se - sb;
  unsigned nmax = __reduce_max_sync(0xFFFFFFFFu, slot < n_slots ? sn : 0u);
  if (slot >= n_slots) return;
  double x[kBatch];
#pragma unroll
  for (int j = 0; j < kBatch; j++) {
    x[j] = 0.0;
    if ((uint32_t)j < sn) x[j] = kIds ? __ldg(contrib + __ldg(ids + sb + j)) : __ldg(contrib + sb + j);
  }
  double v = plus_zero_sum(x[0]);
#pragma unroll
  for (int j = 1; j < kBatch; j++) {
    if ((unsigned)j >= nmax) break;  // warp-uniform
    const double t = v + x[j];
    v = (uint32_t)j < sn ? t : v;
  }
  for (uint32_t k = sb + kBatch; k < se; k++) v += kIds ? contrib[ids[k]] : contrib[k];
  out[slot] = v;
}

// Sparse block products of the Newton iteration (FESolver.cpp:454-466):
// one thread per output entry walks its precomputed list in the reference's
// order; explicit _rn operations keep (K x) coef and the running sum from
// being fused, so each entry is the reference's value bit for bit (structural
// zeros, which the reference's symmetric product also visits, add +-0 there
// and are not visited here).
__global__ void block_mv_kernel(const BlockMvArgs a) {
  const uint64_t r = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= a.n_out) return;
  double acc = a.y[r];
  const uint32_t e = __ldg(a.ptr + r + 1);
  for (uint32_t k = __ldg(a.ptr + r); k < e; k++) {
    const double xv = a.x[__ldg(a.xi + k)];
    if (a.sym && !(fabs(xv) > 1e-20)) continue;
    acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(__ldg(a.K + __ldg(a.slot + k)), xv), a.coef));
  }
  a.y[r] = acc;
}

__global__ void linear_mpc_kernel(const LinearMpcArgs a) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  a.F[a.eq[k] - 1] = a.b[k];
  for (uint32_t t = a.ptr[k]; t < a.ptr[k + 1]; t++) a.K[a.slot[t]] += a.coef[t];
}

// Rigid-body MPC rows (RigidBodyMpc::update, Mpc.cpp:70-164, and
// FEStorage.cpp:51-61): one thread per MPC equation.
__global__ void mpc_kernel(const MpcArgs a) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n_mpc) return;
  const uint32_t* me = a.master_eq6 + (uint64_t)k * 6;
  const double w0[3] = {a.U[me[0] - 1], a.U[me[1] - 1], a.U[me[2] - 1]};
  const double th[3] = {a.U[me[3] - 1], a.U[me[4] - 1], a.U[me[5] - 1]};
  const double tn = sqrt(th[0] * th[0] + th[1] * th[1] + th[2] * th[2]);
  double c1, c2, c3, c4;
  if (tn < 1.0e-3) {
    c1 = 1.0;
    c2 = 0.5;
    c3 = -1.0 / 3.0;
    c4 = -1.0 / 12.0;
  } else {
    const double sn = sin(tn), cs = cos(tn);
    c1 = sn / tn;
    c2 = (1.0 - cs) / (tn * tn);
    c3 = (tn * cs - sn) / (tn * tn * tn);
    c4 = (tn * sn - 2.0 + 2.0 * cs) / (tn * tn * tn * tn);
  }
  // Levi-Civita e_{i m j} with the reference's table (solidmech.h:24-33)
  auto lc = [](int i, int m, int j) -> double {
    if (i == m || m == j || i == j) return 0.0;
    return ((i == 0 && m == 1 && j == 2) || (i == 1 && m == 2 && j == 0) ||
            (i == 2 && m == 0 && j == 1))
               ? 1.0
               : -1.0;
  };
  const int i = a.slave_dof[k];
  const double ct = cos(tn);
  double Crow[3];
  for (int j = 0; j < 3; j++) {
    const double tm = lc(i, 0, j) * th[0] + lc(i, 1, j) * th[1] + lc(i, 2, j) * th[2];
    Crow[j] = ct * (i == j ? 1.0 : 0.0) + c1 * tm + c2 * th[i] * th[j];
  }
  const double* mp = a.xyz + (uint64_t)(a.master[k] - 1) * 3;
  const double* sp = a.xyz + (uint64_t)(a.slave[k] - 1) * 3;
  const double pq[3] = {sp[0] - mp[0], sp[1] - mp[1], sp[2] - mp[2]};
  double cD[3][3];
  for (int j = 0; j < 3; j++)
    for (int l = 0; l < 3; l++) {
      const double Iij = i == j ? 1.0 : 0.0, Iil = i == l ? 1.0 : 0.0, Ijl = j == l ? 1.0 : 0.0;
      cD[j][l] = Iij * (-c1) * th[l] +
                 c3 * th[l] * (lc(i, 0, j) * th[0] + lc(i, 1, j) * th[1] + lc(i, 2, j) * th[2]) +
                 c1 * lc(i, l, j) + c4 * th[l] * th[i] * th[j] + c2 * (Iil * th[j] + th[i] * Ijl);
    }
  const double b = w0[i] + (Crow[0] - (i == 0)) * pq[0] + (Crow[1] - (i == 1)) * pq[1] +
                   (Crow[2] - (i == 2)) * pq[2] - a.U[a.slave_eq[k] - 1];
  const uint32_t* sl = a.slot + (uint64_t)k * 5;
  a.K[sl[0]] += 1.0;
  a.K[sl[1]] += -1.0;
  for (int l = 0; l < 3; l++)
    a.K[sl[2 + l]] += -(cD[0][l] * pq[0] + cD[1][l] * pq[1] + cD[2][l] * pq[2]);
  a.F[a.eq[k] - 1] = b;
}

// TETRA0 (TETRA0.cpp:18-78, 110-199) and QUADTH (QUADTH.cpp:22-49): one
// thread per element; contributions in Element::assembleK order.
__device__ double det4_lu(double* m) {
  double det = 1.0;
  for (int k = 0; k < 4; k++) {
    int p = k;
    double best = fabs(m[k * 4 + k]);
    for (int i = k + 1; i < 4; i++) {
      const double v = fabs(m[i * 4 + k]);
      if (v > best) {
        best = v;
        p = i;
      }
    }
    if (best == 0.0) return 0.0;
    if (p != k) {
      for (int j = 0; j < 4; j++) {
        const double t = m[k * 4 + j];
        m[k * 4 + j] = m[p * 4 + j];
        m[p * 4 + j] = t;
      }
      det = -det;
    }
    const double piv = m[k * 4 + k];
    det *= piv;
    for (int i = k + 1; i < 4; i++) {
      const double f = m[i * 4 + k] / piv;
      for (int j = k + 1; j < 4; j++) m[i * 4 + j] -= f * m[k * 4 + j];
    }
  }
  return det;
}

__global__ void linear_kernel(const LinearArgs a) {
  const uint32_t e = a.e_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.n_elems) return;
  const uint32_t* c = a.conn + (uint64_t)e * 4;
  double P[4][3];
  for (int n = 0; n < 4; n++)
    for (int d = 0; d < 3; d++) P[n][d] = a.xyz[(uint64_t)(c[n] - 1) * 3 + d];
  if (a.etype == 3) {
    double S[16];
    for (int n = 0; n < 4; n++) {
      S[n * 4 + 0] = 1.0;
      S[n * 4 + 1] = P[n][0];
      S[n * 4 + 2] = P[n][1];
      S[n * 4 + 3] = P[n][2];
    }
    const double vol = det4_lu(S) / 6.0;
    if (!(vol > 0.0)) flag_element(a.status, e + 1);
    const double Em = a.eparams[kEparamStride * (uint64_t)e];
    const double my = a.eparams[kEparamStride * (uint64_t)e + 1];
    const double Ac = Em / ((1. + my) * (1. - 2. * my));
    // C (6x6, makeC) as dense
    double Cm[6][6] = {};
    Cm[0][0] = Cm[1][1] = Cm[2][2] = (1. - my) * Ac;
    Cm[0][1] = Cm[1][0] = Cm[0][2] = Cm[2][0] = Cm[1][2] = Cm[2][1] = my * Ac;
    Cm[3][3] = Cm[4][4] = Cm[5][5] = (1. / 2. - my) * Ac;
    // makeB: b, c, d coefficients
    auto X = [&](int n, int d) { return P[n][d]; };
    const double x12 = X(0, 0) - X(1, 0), x13 = X(0, 0) - X(2, 0), x14 = X(0, 0) - X(3, 0);
    const double x23 = X(1, 0) - X(2, 0), x24 = X(1, 0) - X(3, 0), x34 = X(2, 0) - X(3, 0);
    const double y12 = X(0, 1) - X(1, 1), y13 = X(0, 1) - X(2, 1), y14 = X(0, 1) - X(3, 1);
    const double y23 = X(1, 1) - X(2, 1), y24 = X(1, 1) - X(3, 1), y34 = X(2, 1) - X(3, 1);
    const double z12 = X(0, 2) - X(1, 2), z13 = X(0, 2) - X(2, 2), z14 = X(0, 2) - X(3, 2);
    const double z23 = X(1, 2) - X(2, 2), z24 = X(1, 2) - X(3, 2), z34 = X(2, 2) - X(3, 2);
    const double x21 = -x12, x31 = -x13, x32 = -x23, x42 = -x24, x43 = -x34;
    const double y21 = -y12, y31 = -y13, y32 = -y23, y42 = -y24, y43 = -y34;
    const double z21 = -z12, z31 = -z13, z32 = -z23, z42 = -z24, z43 = -z34;
    const double bb[4] = {y42 * z32 - y32 * z42, y31 * z43 - y34 * z13, y24 * z14 - y14 * z24,
                          y13 * z21 - y12 * z31};
    const double cc[4] = {x32 * z42 - x42 * z32, x43 * z31 - x13 * z34, x14 * z24 - x24 * z14,
                          x21 * z13 - x31 * z12};
    const double dd[4] = {x42 * y32 - x32 * y42, x31 * y43 - x34 * y13, x24 * y14 - x14 * y24,
                          x13 * y21 - x12 * y31};
    const double Af = -1. / 6. / vol;
    double B[6][12] = {};
    for (int i = 0; i < 4; i++) {
      B[0][3 * i + 0] = bb[i] * Af;
      B[1][3 * i + 1] = cc[i] * Af;
      B[2][3 * i + 2] = dd[i] * Af;
      B[3][3 * i + 0] = cc[i] * Af;
      B[3][3 * i + 1] = bb[i] * Af;
      B[4][3 * i + 1] = dd[i] * Af;
      B[4][3 * i + 2] = cc[i] * Af;
      B[5][3 * i + 0] = dd[i] * Af;
      B[5][3 * i + 2] = bb[i] * Af;
    }
    int idx = 0;
    for (int r = 0; r < 12; r++)
      for (int col = r; col < 12; col++, idx++) {
        double v = 0.0;
        for (int k = 0; k < 6; k++) {
          double cb = 0.0;
          for (int l = 0; l < 6; l++) cb += Cm[k][l] * B[l][col];
          v += B[k][r] * cb;
        }
        const uint64_t i = (uint64_t)e * 78 + idx;
        a.contribK[a.kpos ? a.kpos[i] : i] = v * vol;
      }
  } else {
    // QUADTH: 2x2 Gauss (isoparametric.h:80-85), conduction k and volume flux
    // (QUADTH.cpp:22-49), capacity rho c for transient analysis (:51-67)
    const double* ep = a.eparams + kEparamStride * (uint64_t)e;
    const double kc = ep[0], vflux = ep[1], rho = ep[2], cap = ep[3];
    double Ke[10] = {}, Ce[10] = {}, Fe[4] = {};
    for (int g = 0; g < 4; g++) {
      const double r = (g & 1) ? kGaussA : -kGaussA;
      const double s = (g & 2) ? kGaussA : -kGaussA;
      const double dN[4][2] = {{-0.25 * (1.0 - s), -0.25 * (1.0 - r)},
                               {+0.25 * (1.0 - s), -0.25 * (1.0 + r)},
                               {+0.25 * (1.0 + s), +0.25 * (1.0 + r)},
                               {-0.25 * (1.0 + s), +0.25 * (1.0 - r)}};
      const double N[4] = {0.25 * (1.0 - r) * (1.0 - s), 0.25 * (1.0 + r) * (1.0 - s),
                           0.25 * (1.0 + r) * (1.0 + s), 0.25 * (1.0 - r) * (1.0 + s)};
      double J[2][2] = {};
      for (int n = 0; n < 4; n++)
        for (int i = 0; i < 2; i++)
          for (int j = 0; j < 2; j++) J[i][j] += dN[n][i] * P[n][j];
      const double det = J[0][0] * J[1][1] - J[0][1] * J[1][0];
      if (!(det >= 1.0e-20)) flag_element(a.status, e + 1);
      const double s1 = 1.0 / det;
      const double Ji[2][2] = {{J[1][1] * s1, -J[0][1] * s1}, {-J[1][0] * s1, J[0][0] * s1}};
      double G[4][2];
      for (int n = 0; n < 4; n++)
        for (int i = 0; i < 2; i++) G[n][i] = Ji[i][0] * dN[n][0] + Ji[i][1] * dN[n][1];
      const double w = 1.0 * det;
      int idx = 0;
      for (int i = 0; i < 4; i++)
        for (int j = i; j < 4; j++, idx++) {
          Ke[idx] += (G[i][0] * kc * G[j][0] + G[i][1] * kc * G[j][1]) * w;
          Ce[idx] = __dadd_rn(Ce[idx], __dmul_rn(N[i] * N[j] * rho * cap, w));
        }
      if (vflux != 0.0)
        for (int i = 0; i < 4; i++) Fe[i] = __dadd_rn(Fe[i], __dmul_rn(N[i], vflux * w));
    }
    for (int i = 0; i < 10; i++) {
      const uint64_t k = (uint64_t)e * 10 + i;
      a.contribK[a.kpos ? a.kpos[k] : k] = Ke[i];
      if (a.contribC) a.contribC[a.kpos ? a.kpos[k] : k] = Ce[i];
    }
    for (int i = 0; i < 4; i++) {
      const uint64_t k = (uint64_t)e * 4 + i;
      a.contribF[a.fpos ? a.fpos[k] : k] = Fe[i];
    }
  }
}

// SurfaceLINETH::buildK (QUADTH.cpp:86-121): 2-point Gauss on the line
// (isoparametric.h:47-50), w = det = length / 2 (isoparametric.cpp:12-26);
// flux: F += N flux w; convection: K += N N^T htc w and F += (N N^T htc w) T_env.
__global__ void line_kernel(const LineArgs a) {
  const uint32_t l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= a.n_lines) return;
  const uint32_t na = a.conn[2 * (uint64_t)l], nb = a.conn[2 * (uint64_t)l + 1];
  double d2 = 0.0;
  for (int k = 0; k < 3; k++) {
    const double d = a.xyz[(uint64_t)(nb - 1) * 3 + k] - a.xyz[(uint64_t)(na - 1) * 3 + k];
    d2 += d * d;
  }
  const double det = sqrt(d2) * 0.5;
  if (!(det > 0.0)) flag_element(a.status, a.first_elem + l);
  const double* par = a.par + 4 * (uint64_t)l;
  const double htc = par[0], flux = par[1], t0 = par[2], t1 = par[3];
  double Ke[3] = {0.0, 0.0, 0.0}, Fe[2] = {0.0, 0.0};
  const double w = 1.0 * det;
  // the flux loop runs over both points before the convection loop, and F
  // takes each product separately (matBVprod, Mat.h), as the reference adds
  if (flux != 0.0)
    for (int g = 0; g < 2; g++) {
      const double r = g ? kGaussA : -kGaussA;
      const double N0 = 0.5 * (1.0 - r), N1 = 0.5 * (1.0 + r);
      Fe[0] = __dadd_rn(Fe[0], __dmul_rn(N0, flux * w));
      Fe[1] = __dadd_rn(Fe[1], __dmul_rn(N1, flux * w));
    }
  if (htc != 0.0)
    for (int g = 0; g < 2; g++) {
      const double r = g ? kGaussA : -kGaussA;
      const double N0 = 0.5 * (1.0 - r), N1 = 0.5 * (1.0 + r);
      const double k00 = N0 * N0 * htc * w, k01 = N0 * N1 * htc * w, k11 = N1 * N1 * htc * w;
      Ke[0] += k00;
      Ke[1] += k01;
      Ke[2] += k11;
      Fe[0] = __dadd_rn(Fe[0], __dmul_rn(k00, t0));
      Fe[0] = __dadd_rn(Fe[0], __dmul_rn(k01, t1));
      Fe[1] = __dadd_rn(Fe[1], __dmul_rn(k01, t0));
      Fe[1] = __dadd_rn(Fe[1], __dmul_rn(k11, t1));
    }
  for (int i = 0; i < 3; i++) {
    const uint64_t k = a.k_off + 3 * (uint64_t)l + i;
    a.contribK[a.kpos ? a.kpos[k] : k] = Ke[i];
  }
  for (int i = 0; i < 2; i++) {
    const uint64_t k = a.f_off + 2 * (uint64_t)l + i;
    a.contribF[a.fpos ? a.fpos[k] : k] = Fe[i];
  }
}

// FMA throughput probe: 8 independent chains per thread, enough warps per SM
// to cover the pipe latency; every result is folded into one store so the
// chains cannot be removed.
template <typename T>
__global__ void fma_probe_kernel(T* out, int iters, T a, T b) {
  T x[8];
#pragma unroll
  for (int k = 0; k < 8; k++) x[k] = (T)(threadIdx.x + k);
  for (int i = 0; i < iters; i++)
#pragma unroll
    for (int k = 0; k < 8; k++) x[k] = x[k] * a + b;
  T s = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) s += x[k];
  if (s == (T)-12345.0) out[0] = s;
}

// One ready flag per device: the table is uploaded once per device (a
// synchronous copy), under a lock so that threads on different devices
// neither race on the flags nor repeat the upload.
constexpr int kMaxTableDevices = 64;
std::atomic<bool> g_tables_ready[kMaxTableDevices];
std::mutex g_tables_mutex;

cudaError_t ensure_tables() {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  if (dev < 0 || dev >= kMaxTableDevices) return cudaErrorInvalidDevice;
  if (g_tables_ready[dev].load(std::memory_order_acquire)) return cudaSuccess;
  std::lock_guard<std::mutex> lock(g_tables_mutex);
  if (g_tables_ready[dev].load(std::memory_order_relaxed)) return cudaSuccess;
  uchar4 h[kKuuPerElem];
  int t = 0;
  for (int i = 0; i < 8; i++)
    for (int di = 0; di < 3; di++)
      for (int j = i; j < 8; j++)
        for (int dj = 0; dj < 3; dj++) {
          if (i == j && dj < di) continue;
          h[t++] = make_uchar4((unsigned char)i, (unsigned char)di, (unsigned char)j,
                               (unsigned char)dj);
        }
  err = cudaMemcpyToSymbol(c_kuu_entry, h, sizeof(h));
  if (err != cudaSuccess) return err;
  // D[(i,k), a, b] -> assemble3 position (see c_dpos)
  int tpos[8][3][8][3];
  for (int u = 0; u < kKuuPerElem; u++) tpos[h[u].x][h[u].y][h[u].z][h[u].w] = u;
  uint16_t dp[kDpos];
  for (int a = 0; a < 8; a++)
    for (int i = 0; i < 3; i++)
      for (int k = i; k < 3; k++)
        for (int b = 0; b < 8; b++) {
          const int at = (a * 6 + hblock(i, k)) * 8 + b;
          if (a <= b) dp[at] = (uint16_t)tpos[a][i][b][k];
          else dp[at] = i == k ? (uint16_t)0xFFFF : (uint16_t)tpos[b][k][a][i];
        }
  err = cudaMemcpyToSymbol(c_dpos, dp, sizeof(dp));
  if (err != cudaSuccess) return err;
  // FP64 kernel: node 7's column and block (derived) and the other entries
  // (owned); the column's 63 rows come first, the block's 6 after them
  uint16_t own[kKuuOwned], der[kKuuDerived * 8];
  int no = 0, nd = 0, nc = kKuuColumn;
  for (int u = 0; u < kKuuPerElem; u++) {
    const int a = h[u].x, i = h[u].y, b = h[u].z, k = h[u].w;
    if (b == 7 && a < 7) {
      uint16_t* row = der + 8 * nd++;
      row[0] = (uint16_t)u;
      for (int bb = 0; bb < 7; bb++)   // K(a,i; bb,k) by its assemble3 position
        row[1 + bb] = (uint16_t)(a < bb ? tpos[a][i][bb][k]
                                 : a > bb ? tpos[bb][k][a][i]
                                 : (i <= k ? tpos[a][i][a][k] : tpos[a][k][a][i]));
    } else if (b == 7 && a == 7) {
      if (nc >= kKuuDerived) return cudaErrorInvalidValue;
      uint16_t* row = der + 8 * nc++;
      row[0] = (uint16_t)u;
      for (int aa = 0; aa < 7; aa++)   // K(aa,i; 7,k): node 7's column, formed first
        row[1 + aa] = (uint16_t)tpos[aa][i][7][k];
    } else {
      own[no++] = (uint16_t)u;
    }
  }
  if (no != kKuuOwned || nd != kKuuColumn || nc != kKuuDerived) return cudaErrorInvalidValue;
  err = cudaMemcpyToSymbol(c_kuu_owned, own, sizeof(own));
  if (err == cudaSuccess) err = cudaMemcpyToSymbol(c_kuu_derived, der, sizeof(der));
  if (err == cudaSuccess) g_tables_ready[dev].store(true, std::memory_order_release);
  return err;
}

}  // namespace

size_t solid81_smem_bytes_wpb(bool mixed, int wpb) {
  const size_t head = mixed ? kDposBytes : kHead64Bytes;
  return head + wpb * (mixed ? sizeof(WarpSmem<float>) : sizeof(WarpSmem<double>));
}

size_t solid81_smem_bytes(bool mixed) { return solid81_smem_bytes_wpb(mixed, kWarpsPerBlock); }

template <typename TT>
void* solid81_fn(int wpb) {
  switch (wpb) {
    case 2: return (void*)solid81_kernel<TT, 2>;
    case 8: return (void*)solid81_kernel<TT, 8>;
    default: return (void*)solid81_kernel<TT, 4>;
  }
}

cudaError_t prepare_device_tables() { return ensure_tables(); }

int solid81_max_blocks_per_sm(bool mixed, int wpb) {
  void* fn = mixed ? solid81_fn<float>(wpb) : solid81_fn<double>(wpb);
  const size_t smem = solid81_smem_bytes_wpb(mixed, wpb);
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
      cudaSuccess)
    return 0;
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, wpb * 32, smem) != cudaSuccess)
    return 0;
  return per_sm;
}

cudaError_t launch_solid81_shaped(const Solid81Args& a, bool mixed, Solid81Shape shape,
                                  cudaStream_t s) {
  if (a.n_elems <= a.e_begin) return cudaSuccess;  // empty element range
  const int wpb = (shape.warps_per_block == 2 || shape.warps_per_block == 8)
                      ? shape.warps_per_block : 4;
  cudaError_t err = ensure_tables();
  if (err != cudaSuccess) return err;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t smem = solid81_smem_bytes_wpb(mixed, wpb);
  const int max_per_sm = solid81_max_blocks_per_sm(mixed, wpb);
  if (max_per_sm < 1) return cudaErrorInvalidConfiguration;
  int per_sm = shape.blocks_per_sm;
  if (per_sm <= 0 || per_sm > max_per_sm) per_sm = max_per_sm;
  const uint64_t quads = ((uint64_t)a.n_elems + kEPW - 1) / kEPW - a.e_begin / kEPW;
  uint64_t blocks = (uint64_t)sms * per_sm;
  const uint64_t need = (quads + wpb - 1) / wpb;
  if (blocks > need) blocks = need;
  const dim3 grid((unsigned)blocks), block(wpb * 32);
  if (mixed) {
    if (wpb == 2) solid81_kernel<float, 2><<<grid, block, smem, s>>>(a);
    else if (wpb == 8) solid81_kernel<float, 8><<<grid, block, smem, s>>>(a);
    else solid81_kernel<float, 4><<<grid, block, smem, s>>>(a);
  } else {
    if (wpb == 2) solid81_kernel<double, 2><<<grid, block, smem, s>>>(a);
    else if (wpb == 8) solid81_kernel<double, 8><<<grid, block, smem, s>>>(a);
    else solid81_kernel<double, 4><<<grid, block, smem, s>>>(a);
  }
  return cudaGetLastError();
}

cudaError_t launch_solid81_jacobian(const JacobianArgs& a, cudaStream_t s) {
  const uint64_t n = (uint64_t)a.n_elems * 8;
  if (n == 0) return cudaSuccess;
  const int bs = 256;
  solid81_jacobian_kernel<<<(unsigned)((n + bs - 1) / bs), bs, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_solid81(const Solid81Args& a, bool mixed, int blocks_per_sm_hint,
                           cudaStream_t s) {
  Solid81Shape shape;
  shape.warps_per_block = kWarpsPerBlock;
  shape.blocks_per_sm = blocks_per_sm_hint;
  return launch_solid81_shaped(a, mixed, shape, s);
}

cudaError_t probe_fma_peak(bool fp64, double* flops) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  void* buf = nullptr;
  cudaError_t e = cudaMalloc(&buf, 16);
  if (e != cudaSuccess) return e;
  const int threads = 512, blocks = sms * 4;
  const int iters = fp64 ? 4096 : 65536;
  cudaEvent_t t0, t1;
  cudaEventCreate(&t0);
  cudaEventCreate(&t1);
  float best = 1e30f;
  for (int rep = 0; rep < 4; rep++) {
    cudaEventRecord(t0);
    if (fp64)
      fma_probe_kernel<double><<<blocks, threads>>>((double*)buf, iters, 0.999999, 1e-7);
    else
      fma_probe_kernel<float><<<blocks, threads>>>((float*)buf, iters, 0.9999f, 1e-7f);
    cudaEventRecord(t1);
    e = cudaEventSynchronize(t1);
    if (e != cudaSuccess) break;
    float ms = 0;
    cudaEventElapsedTime(&ms, t0, t1);
    if (rep > 0 && ms < best) best = ms;
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  cudaFree(buf);
  *flops = 2.0 * 8.0 * (double)iters * threads * blocks / (best * 1e-3);
  return e;
}

cudaError_t launch_gather_bs(const GatherArgs& a, int bs, cudaStream_t s) {
  if (a.n_slots <= a.s_begin) return cudaSuccess;
  if (bs != 128 && bs != 256 && bs != 512 && bs != 1024) bs = 256;
  gather_sorted_kernel<true><<<(unsigned)((a.n_slots - a.s_begin + bs - 1) / bs), bs, 0, s>>>(
      a.s_begin, a.n_slots, a.ptr, a.ids, a.contrib, a.out, a.skip);
  return cudaGetLastError();
}

cudaError_t launch_gather(const GatherArgs& a, cudaStream_t s) { return launch_gather_bs(a, 256, s); }

cudaError_t launch_segsum(const SegSumArgs& a, int bs, cudaStream_t s) {
  if (a.n_slots <= a.s_begin) return cudaSuccess;
  if (bs != 128 && bs != 256 && bs != 512 && bs != 1024) bs = 256;
  gather_sorted_kernel<false><<<(unsigned)((a.n_slots - a.s_begin + bs - 1) / bs), bs, 0, s>>>(
      a.s_begin, a.n_slots, a.ptr, nullptr, a.contrib, a.out, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_block_mv(const BlockMvArgs& a, cudaStream_t s) {
  if (a.n_out == 0) return cudaSuccess;
  const int bs = 128;
  block_mv_kernel<<<(unsigned)((a.n_out + bs - 1) / bs), bs, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_linear_mpc(const LinearMpcArgs& a, cudaStream_t s) {
  if (a.n == 0) return cudaSuccess;
  const int bs = 128;
  linear_mpc_kernel<<<(a.n + bs - 1) / bs, bs, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_mpc(const MpcArgs& a, cudaStream_t s) {
  if (a.n_mpc == 0) return cudaSuccess;
  const int bs = 128;
  mpc_kernel<<<(a.n_mpc + bs - 1) / bs, bs, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_lines(const LineArgs& a, cudaStream_t s) {
  if (a.n_lines == 0) return cudaSuccess;
  const int bs = 128;
  line_kernel<<<(a.n_lines + bs - 1) / bs, bs, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_linear(const LinearArgs& a, cudaStream_t s) {
  if (a.n_elems <= a.e_begin) return cudaSuccess;
  const int bs = 128;
  linear_kernel<<<(a.n_elems - a.e_begin + bs - 1) / bs, bs, 0, s>>>(a);
  return cudaGetLastError();
}

// PLANE41 algebra (PLANE41.cpp:29-101): with B = B_L + Omega B_omega (3x8),
//   Kuu += (2 B^T Dd B + B_omega^T S4 B_omega) w,  Kup += B^T Dp w,
//   Kpp -= w / k,  Qe += B^T S w,  Fp += (J - 1 - p/k) w,
// Dd and Dp the (XX, YY, XY) part of getDdDp_UP with C_zz = 1; K and F take
// -Qe, -Fp and the entries in ElementPLANE41::assembleK order (PLANE41.h:54-95).
__global__ void plane41_kernel(const Plane41Args a) {
  const uint32_t e = a.e_begin + blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= a.n_elems) return;
  const uint32_t* cn = a.conn + (uint64_t)e * 4;
  double X[4][2];
  uint32_t eq[4][2];
  for (int n = 0; n < 4; n++) {
    X[n][0] = a.xyz[(uint64_t)(cn[n] - 1) * 3 + 0];
    X[n][1] = a.xyz[(uint64_t)(cn[n] - 1) * 3 + 1];
    eq[n][0] = a.node_eq3[(uint64_t)(cn[n] - 1) * 4 + 0];
    eq[n][1] = a.node_eq3[(uint64_t)(cn[n] - 1) * 4 + 1];
  }
  const uint32_t peq = a.p_eq[e];
  const double pc = a.U_cur[peq - 1];
  const double ps = a.have_state ? a.U_state[peq - 1] : 0.0;
  int mat_id = a.mat_id;
  const double* mc = a.mc;
  double kbulk = a.kbulk;
  if (a.elem_mesh) {
    const double* mm = a.mesh_mat + 8 * (uint64_t)a.elem_mesh[e];
    mat_id = (int)mm[0];
    mc = mm + 1;
    kbulk = mm[6];
  }
  double Us[8];
  for (int n = 0; n < 4; n++)
    for (int d = 0; d < 2; d++) Us[2 * n + d] = a.have_state ? a.U_state[eq[n][d] - 1] : 0.0;
  const int comp[3] = {0, 3, 1};  // M_XX, M_YY, M_XY in the Voigt order xx xy xz yy yz zz
  double Kuu[8][8] = {}, Kup[8] = {}, Qe[8] = {};
  double Kpp = 0.0, Fp = 0.0;
  bool bad = false;
  for (int g = 0; g < 4; g++) {
    // isoparametric quad, 2x2 Gauss (isoparametric.h:80-85, .cpp:13-137)
    const double r = (g & 1) ? kGaussA : -kGaussA;
    const double sg = (g & 2) ? kGaussA : -kGaussA;
    const double dN[4][2] = {{-0.25 * (1.0 - sg), -0.25 * (1.0 - r)},
                             {+0.25 * (1.0 - sg), -0.25 * (1.0 + r)},
                             {+0.25 * (1.0 + sg), +0.25 * (1.0 + r)},
                             {-0.25 * (1.0 + sg), +0.25 * (1.0 - r)}};
    double Jm[2][2] = {};
    for (int n = 0; n < 4; n++)
      for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) Jm[i][j] += dN[n][i] * X[n][j];
    const double det = Jm[0][0] * Jm[1][1] - Jm[0][1] * Jm[1][0];
    if (!(det >= 1.0e-20)) bad = true;
    const double id = 1.0 / det;
    const double Ji[2][2] = {{Jm[1][1] * id, -Jm[0][1] * id}, {-Jm[1][0] * id, Jm[0][0] * id}};
    double G[4][2];
    for (int n = 0; n < 4; n++)
      for (int i = 0; i < 2; i++) G[n][i] = Ji[i][0] * dN[n][0] + Ji[i][1] * dN[n][1];
    const double w = 1.0 * det;
    // state: O = B_omega U (dU/dx, dU/dy, dV/dx, dV/dy), C (xx, yy, xy)
    double O[4] = {0.0, 0.0, 0.0, 0.0};
    for (int n = 0; n < 4; n++) {
      O[0] += G[n][0] * Us[2 * n];
      O[1] += G[n][1] * Us[2 * n];
      O[2] += G[n][0] * Us[2 * n + 1];
      O[3] += G[n][1] * Us[2 * n + 1];
    }
    const double Cxx = 1.0 + 2 * O[0] + O[0] * O[0] + O[2] * O[2];
    const double Cyy = 1.0 + 2 * O[3] + O[3] * O[3] + O[1] * O[1];
    const double Cxy = O[1] + O[2] + O[0] * O[1] + O[2] * O[3];
    const double C6[6] = {Cxx, Cxy, 0.0, Cyy, 0.0, 1.0};
    MatOut<double> mo;
    double wD[21];
    material<double>(mat_id, mc, C6, ps, pc, 1.0, mo, wD);  // wD = 2 Dd
    const double S[3] = {a.have_state ? mo.S[0] : 0.0, a.have_state ? mo.S[3] : 0.0,
                         a.have_state ? mo.S[1] : 0.0};
    double E[3][3];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) E[i][j] = 0.5 * wD[sym6u(comp[i], comp[j])];
    const double det2 = Cxx * Cyy - Cxy * Cxy;  // det C (C_zz = 1)
    const double J = mo.J;
    const double Dp[3] = {J * Cyy / det2, J * Cxx / det2, -J * Cxy / det2};
    if (!(J > 0.0 && isfinite(J))) bad = true;
    // B = B_L + Omega B_omega, rows (xx, yy, xy), columns (node, dof)
    double B[3][8];
    for (int n = 0; n < 4; n++) {
      const double gx = G[n][0], gy = G[n][1];
      B[0][2 * n] = gx + O[0] * gx;
      B[0][2 * n + 1] = O[2] * gx;
      B[1][2 * n] = O[1] * gy;
      B[1][2 * n + 1] = gy + O[3] * gy;
      B[2][2 * n] = gy + O[1] * gx + O[0] * gy;
      B[2][2 * n + 1] = gx + O[3] * gx + O[2] * gy;
    }
    double EB[3][8];
    for (int i = 0; i < 3; i++)
      for (int c = 0; c < 8; c++) EB[i][c] = E[i][0] * B[0][c] + E[i][1] * B[1][c] + E[i][2] * B[2][c];
    for (int r2 = 0; r2 < 8; r2++)
      for (int c = r2; c < 8; c++) {
        double v = 2.0 * (B[0][r2] * EB[0][c] + B[1][r2] * EB[1][c] + B[2][r2] * EB[2][c]);
        // geometric term: B_omega^T S4 B_omega couples equal DoFs only
        if ((r2 & 1) == (c & 1)) {
          const int na = r2 >> 1, nb = c >> 1;
          v += G[na][0] * (S[0] * G[nb][0] + S[2] * G[nb][1]) +
               G[na][1] * (S[2] * G[nb][0] + S[1] * G[nb][1]);
        }
        Kuu[r2][c] += v * w;
      }
    for (int c = 0; c < 8; c++) {
      Kup[c] += (B[0][c] * Dp[0] + B[1][c] * Dp[1] + B[2][c] * Dp[2]) * w;
      Qe[c] += (B[0][c] * S[0] + B[1][c] * S[1] + B[2][c] * S[2]) * w;
    }
    Fp += (J - 1 - pc / kbulk) * w;
    Kpp -= 1.0 / kbulk * w;
  }
  if (bad) flag_element(a.status, e + 1);
  const uint64_t kb = (uint64_t)e * 45, fb = (uint64_t)e * 9;
  auto kd = [&](uint64_t i) { return a.kpos ? (uint64_t)a.kpos[i] : i; };
  auto fd = [&](uint64_t i) { return a.fpos ? (uint64_t)a.fpos[i] : i; };
  int t = 0;
  for (int i = 0; i < 4; i++)
    for (int j = i; j < 4; j++)
      for (int di = 0; di < 2; di++)
        for (int dj = 0; dj < 2; dj++) {
          if (i == j && dj > di) continue;
          const int r2 = 2 * i + di, c = 2 * j + dj;
          a.contribK[kd(kb + t++)] = r2 <= c ? Kuu[r2][c] : Kuu[c][r2];
        }
  for (int c = 0; c < 8; c++) a.contribK[kd(kb + 36 + c)] = Kup[c];
  a.contribK[kd(kb + 44)] = Kpp;
  for (int c = 0; c < 8; c++) a.contribF[fd(fb + c)] = -Qe[c];
  a.contribF[fd(fb + 8)] = -Fp;
}

cudaError_t launch_plane41(const Plane41Args& a, cudaStream_t s) {
  if (a.n_elems <= a.e_begin) return cudaSuccess;
  const int bs = 128;
  plane41_kernel<<<(a.n_elems - a.e_begin + bs - 1) / bs, bs, 0, s>>>(a);
  return cudaGetLastError();
}

__global__ void slot_last_range_kernel(uint64_t n_slots, const uint32_t* ptr, const uint32_t* ids,
                                       uint32_t n_kc, const uint32_t* eb, int n, uint8_t* out) {
  const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_slots) return;
  const uint32_t b = ptr[s], e = ptr[s + 1];
  int r = 0;
  if (e > b) {
    const uint32_t el = ids[e - 1] / n_kc;  // ids ascend within a slot
    while (r + 1 < n && el >= eb[r + 1]) r++;
  }
  out[s] = (uint8_t)r;
}

cudaError_t launch_slot_last_range(uint64_t n_slots, const uint32_t* ptr, const uint32_t* ids,
                                   uint32_t n_kc, const uint32_t* eb, int n, uint8_t* out,
                                   cudaStream_t s) {
  if (n_slots == 0) return cudaSuccess;
  const int bs = 256;
  slot_last_range_kernel<<<(unsigned)((n_slots + bs - 1) / bs), bs, 0, s>>>(n_slots, ptr, ids,
                                                                          n_kc, eb, n, out);
  return cudaGetLastError();
}

}  // namespace nla3d_gpu
