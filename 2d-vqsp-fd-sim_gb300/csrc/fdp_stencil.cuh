// Fused time-stepping kernels for the 2-D velocity-stress Biot poroelastic
// scheme.  The stress phase of a time level (time_loop.F90:93-124) is one
// launch of k_stress, or k_stress_frame beside k_stress_core (frame/core
// split); the velocity phase including the bottom non-reflecting row
// (time_loop.F90:133-179) likewise with k_velocity; k_edge is the one step
// with a cross-column dependency (the stress-imaging row 1,
// hplane_1_velocity.F90:61-76) plus receiver sampling
// (store_seismograms.F90:47-104, store_seismograms_pressure.F90:45-58);
// inside a run of levels the split does that step in the next level's
// k_stress_frame (and the stress samples in k_velocity_frame).
//
// Every row routine of the reference (strain_*, stress_*, inh_*, sto_*)
// becomes a branch on the cell's row and column class inside these kernels;
// the arithmetic of each branch is written in the reference's evaluation
// order and the code is compiled without FMA contraction, so a kernel's
// results equal a serial CPU evaluation of the same routines bit for bit.
//
// Threads: blocks of 32 (x) x 8 (z) threads; a warp spans 32 consecutive
// columns, so every row class is warp-uniform.  The unit kernels give a
// thread kRZS (stress) or kRZV (velocity) consecutive rows of one column;
// the core kernels give a thread four consecutive columns of one row.
//
// Layout (all arrays x-fastest, the reference's column-major order):
//   fields   T[NZ + 2*PADZ][pitch], pointer p.F points at (I=PMLL, L=0)
//   medium   either (table mode) JM int32 in the field layout and a derived
//            per-material table coef[k*cld + jm], or (plane mode) one plane
//            per distinct derived coefficient column in the field layout,
//            with columns that are equal (or equal up to sign) across all
//            materials stored once and columns that are constant folded
//            into the kernel parameters
//   x-PML profiles [L][J] (the reference's own layout), z-PML profiles
//            stored transposed [J][I-PMLL] so a warp reads them coalesced
//   memory variables in the reference's own bounds (ppml.F90:85-112)
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

namespace fdp {

// Derived material coefficients (one column per k, indexed by JM).
// The exponential-integrator factors EXP(-REL3_Q) and
// (REL2/REL3_Q)*(1-EXP(-REL3_Q)) that the reference re-evaluates at every
// cell and step (inh_qx_int.F90:44, inh_v_uv_int.F90:46) depend only on the
// material, so they are evaluated once per material on the host with the
// same expression and C library.
enum Coef {
  C_MU = 0, C_SXX1, C_SXX2, C_SXX3, C_SZZ1, C_SZZ2, C_SZZ3, C_P1, C_P2, C_P3,
  C_EQX, C_CU, C_R1QX, C_R2QX, C_R1U, C_R3U,
  C_EQZ, C_CW, C_R1QZ, C_R2QZ, C_R1W, C_R3W,
  C_AUXW, C_AUXQZ,
  C_NCOEF
};

constexpr int kPadX = 4;
constexpr int kPadZ = 2;
constexpr int kBX = 32;  // block width (cells along x)
// Launch shape of k_stress / k_velocity, fixed at build time: threads per
// block kBX x kBZ and rows per thread kRZS (stress) and kRZV (velocity).
// Measured on the layered 2048^2 workload (FP32, per-cell Biot planes):
// one row per thread suits the stress phase (40 registers, 75 % occupancy),
// four rows with a register window suit the velocity phase, with its
// registers capped at three FP32 blocks (two FP64 blocks) per SM.
#ifndef FDP_KBZ
#define FDP_KBZ 8
#endif
#ifndef FDP_KRZS
#define FDP_KRZS 1
#endif
#ifndef FDP_KRZV
#define FDP_KRZV 4
#endif
#ifndef FDP_MIN_BLOCKS_F32
#define FDP_MIN_BLOCKS_F32 3
#endif
#ifndef FDP_MIN_BLOCKS_F64
#define FDP_MIN_BLOCKS_F64 2
#endif
constexpr int kBZ = FDP_KBZ;  // block height (threads along z)
constexpr int kRZS = FDP_KRZS;
constexpr int kRZV = FDP_KRZV;
#define FDP_VELOCITY_BOUNDS(T) __launch_bounds__(kBX * kBZ, sizeof(T) == 4 ? FDP_MIN_BLOCKS_F32 : FDP_MIN_BLOCKS_F64)
static_assert(kBZ * kRZS >= 5, "the first block row of k_stress must hold rows 0..4");

enum MediumMode { M_TABLE = 0, M_PLANES = 1, M_BIOT = 2 };

// Plane mode whose columns follow Biot's relations (M_BIOT): five planes per
// phase, with the aliases resolved at compile time.  Slots 0..4 are the
// stress planes MU, SIG_XX_1 (= SIG_ZZ_2), SIG_XX_2 (= SIG_ZZ_1),
// SIG_XX_3 (= SIG_ZZ_3 = -PRES_1 = -PRES_2), PRES_3; slots 5..9 the velocity
// planes EXP(-REL3_Q), the drag factor, REL1_Q (= REL3_U), REL2_Q, REL1_U.
// The host selects this mode only after checking, column by column, that
// the medium's derived coefficients have exactly these equalities.
__host__ __device__ constexpr int biot_slot(int k) {
  return k == 0 ? 0 : k == 1 ? 1 : k == 2 ? 2 : k == 3 ? 3 : k == 4 ? 2 : k == 5 ? 1 : k == 6 ? 3 : k == 7 ? 3
       : k == 8 ? 3 : k == 9 ? 4 : k == 10 ? 5 : k == 11 ? 6 : k == 12 ? 7 : k == 13 ? 8 : k == 14 ? 9
       : k == 15 ? 7 : k == 16 ? 5 : k == 17 ? 6 : k == 18 ? 7 : k == 19 ? 8 : k == 20 ? 9 : k == 21 ? 7 : -1;
}
__host__ __device__ constexpr bool biot_neg(int k) { return k == 7 || k == 8; }

template <class T> struct Params {
  int MX, MZ, TPML, PMLL, PMLXH, PMLZH, NX, NZ, MX1, LIN_X, LIN_Z;
  int pitch;    // field row pitch in elements
  // core rectangles [x0, x1) x [z0, z1) of each phase (stress excluding row
  // LIN_Z), updated by the vectorised core kernels; the unit kernels then
  // skip them.  Empty (x0 == x1) when the unit kernels update every cell.
  int cs_x0, cs_x1, cs_z0, cs_z1, cv_x0, cv_x1, cv_z0, cv_z1;
  T AH, BH, CH, BC, A, B, DT, DTE;
  // the wavefield a kernel reads (UM..PRES) and the arrays it writes its
  // phase's new values to (oUM..oPRES): the same arrays when levels update
  // in place, the other buffer of each pair when they alternate
  T *UM, *WM, *QX, *QZ, *TXX, *TZZ, *TXZ, *PRES;
  T *oUM, *oWM, *oQX, *oQZ, *oTXX, *oTZZ, *oTXZ, *oPRES;
  // the stress core rectangle includes the source row LIN_Z (its update adds
  // the source term); else the source row is left to the unit kernels
  int cs_src;
  // medium, table mode
  const int32_t* JM;
  const T* coef;
  long long cld;
  // medium, plane mode: coefficient k is cval[k] when src[k] < 0, else plane
  // src[k] (negated when neg[k]) at the cell's field offset
  const T* planes;
  long long pstride;
  const T* cptr[C_NCOEF];  // plane of coefficient k at (PMLL, 0), or null when constant
  const T* bplane[10];     // M_BIOT: the plane of each slot at (PMLL, 0)
  int src[C_NCOEF];
  int neg[C_NCOEF];
  T cval[C_NCOEF];
  const T* AUX;  // [2][NX]: AUXIL_W and AUXIL_QZ of JM(I,0), for the imaging row 1
  // x-PML profiles, [L][J]: OD* with J in 0..TPML, OD2* with J in 0..TPML+1
  const T *ODA_XL, *ODB_XL, *ODC_XL, *ODD_XL, *ODA_XH, *ODB_XH, *ODC_XH, *ODD_XH;
  const T *ODA2_XL, *ODB2_XL, *ODC2_XL, *ODD2_XL, *ODA2_XH, *ODB2_XH, *ODC2_XH, *ODD2_XH;
  // z-PML profiles, [J][I-PMLL]
  const T *ODA_ZH, *ODB_ZH, *ODC_ZH, *ODD_ZH, *ODA2_ZH, *ODB2_ZH, *ODC2_ZH, *ODD2_ZH;
  // memory variables (reference bounds)
  T *PZXL, *PZXH, *PXXL, *PXXH, *OXXL, *OXXH, *PXZH, *PZZH, *OZZH;
  T *RXXL, *RXXH, *SXXL, *SXXH, *RZXL, *RZXH, *GXXL, *GXXH, *HXXL, *HXXH, *GZXL, *GZXH;
  T *RXZH, *GXZH, *RZZH, *SZZH, *GZZH, *HZZH;
  // bottom non-reflecting row: AB[0..7] = ABW01..ABW22, AB[8..15] = ABH01..ABH22
  const T* AB;
  T* HIST;  // [4][3][NX]: SZ_U, SZ_W, SZ_QX, SZ_QZ; row k = TIKMZk
  // source
  const T* STF;
  int MT2;
  const int* it_base;
  // receivers: REC[4*j..] = IRECX LRECX IRECZ LRECZ; RAW[(it-1)*MR*6 + j*6 + c]
  int MR;
  const int* REC;
  T* RAW;
  // device status word: bit 0 set when a bounded wait gave up
  int* err;
};

#define FDP_F(ptr, I, L) (ptr)[(long long)(L) * p.pitch + ((I) - p.PMLL)]
// read-only load through the non-coherent path, for arrays no thread of the
// running kernel writes (velocities in k_stress, stresses in k_velocity)
#define FDP_R(ptr, I, L) __ldg(&FDP_F(ptr, I, L))

// Material coefficient k of the cell at field offset `cell` (material J in
// table mode).  Negation is exact, so a plane shared up to sign returns the
// reference's value bit for bit.
template <class T, int MODE>
__device__ __forceinline__ T coef(const Params<T>& p, int k, long long cell, int J) {
  if (MODE == M_TABLE) return __ldg(p.coef + (long long)k * p.cld + J);
  if (MODE == M_BIOT) {
    const T v = __ldg(p.bplane[biot_slot(k)] + cell);
    return biot_neg(k) ? -v : v;
  }
  const T* c = p.cptr[k];
  if (!c) return p.cval[k];
  const T v = __ldg(c + cell);
  return p.neg[k] ? -v : v;
}
#define FDP_C(k) coef<T, MODE>(p, (k), cell_, J_)

// ---------------------------------------------------------------------------
// Interior fast paths.  A thread of k_stress (k_velocity) updates kRZS
// (kRZV) consecutive rows of one column, and a warp 32 consecutive columns
// of those rows.  When every row is an interior row (2..MZ-2, not the source row) and
// all 32 columns lie where every stencil of the phase is the 4th-order one,
// the warp runs these straight-line versions of the interior branches of
// stress_cell / velocity_cell (same expressions, same order) without region
// tests.  The column's values that the z stencils of those rows share are
// loaded once, into a window of kRZS + 3 (kRZV + 3) registers per field.

// stress: EXX needs 3 <= I <= MX-2 (strain_uw_xx.F90:80); EXZ, EZZ, the
// stresses cover that range
template <class T>
__device__ __forceinline__ bool stress_fast_rows(const Params<T>& p, int I, int L0) {
  const int I0 = I - (int)(threadIdx.x & 31);
  const int L1 = L0 + kRZS - 1;
  return L0 >= 2 && L1 <= p.MZ - 2 && (p.LIN_Z < L0 || p.LIN_Z > L1) && I0 >= 3 && I0 + 31 <= p.MX - 2;
}

template <class T, int MODE>
__device__ __forceinline__ void stress_interior_rows(const Params<T>& p, int I, int L0) {
  const long long P = p.pitch;
  const long long c0 = (long long)L0 * P + (I - p.PMLL);
  const T* U = p.UM + c0;
  const T* W = p.WM + c0;
  const T* X = p.QX + c0;
  const T* Z = p.QZ + c0;
  // u[k] = U(I, L0-2+k); w[k], z[k] = W, QZ(I, L0-1+k)
  T u[kRZS + 3], w[kRZS + 3], z[kRZS + 3];
#pragma unroll
  for (int k = 0; k < kRZS + 3; ++k) {
    u[k] = __ldg(U + (k - 2) * P);
    w[k] = __ldg(W + (k - 1) * P);
    z[k] = __ldg(Z + (k - 1) * P);
  }
  // the stresses of all rows; they receive the new values
  T oxz[kRZS], oxx[kRZS], ozz[kRZS], opr[kRZS];
#pragma unroll
  for (int r = 0; r < kRZS; ++r) {
    oxz[r] = p.TXZ[c0 + r * P]; oxx[r] = p.TXX[c0 + r * P];
    ozz[r] = p.TZZ[c0 + r * P]; opr[r] = p.PRES[c0 + r * P];
  }
#pragma unroll
  for (int r = 0; r < kRZS; ++r) {
    const long long cell_ = c0 + r * P;
    const int J_ = (MODE == M_TABLE) ? p.JM[cell_] : 0;
    const T* Ur = U + r * P;
    const T* Wr = W + r * P;
    const T* Xr = X + r * P;
    // strain_uw_xz.F90:81-84
    const T exz = p.AH * (u[r + 3] - u[r] + __ldg(Wr + 1) - __ldg(Wr - 2))
                + p.BH * (u[r + 2] - u[r + 1] + w[r + 1] - __ldg(Wr - 1));
    // strain_uw_zz.F90:51,58-59 and strain_q_zz.F90:48,55-56
    T ezz = (p.CH * (w[r + 2] - w[r + 1]));
    ezz = p.AH * (w[r + 3] - w[r]) + p.BC * ezz;
    T qzz = (p.CH * (z[r + 2] - z[r + 1]));
    qzz = p.AH * (z[r + 3] - z[r]) + p.BC * qzz;
    // strain_uw_xx.F90:82-83 and strain_q_xx.F90:77-78
    const T exx = p.AH * (__ldg(Ur + 2) - __ldg(Ur - 1)) + p.BH * (__ldg(Ur + 1) - u[r + 2]);
    const T qxx = p.AH * (__ldg(Xr + 2) - __ldg(Xr - 1)) + p.BH * (__ldg(Xr + 1) - __ldg(Xr));
    // stress_xz.F90:44-46 and stress_nn.F90:53-59
    const T TXZv = FDP_C(C_MU) * exz;
    oxz[r] = oxz[r] + p.DTE * TXZv;
    const T s1 = FDP_C(C_SXX1), s2 = FDP_C(C_SXX2), s3 = FDP_C(C_SXX3);
    const T z1 = FDP_C(C_SZZ1), z2 = FDP_C(C_SZZ2), z3 = FDP_C(C_SZZ3);
    const T q1 = FDP_C(C_P1), q2 = FDP_C(C_P2), q3 = FDP_C(C_P3);
    const T TXXv = s1 * exx + s2 * ezz + s3 * qxx + s3 * qzz;
    const T TZZv = z1 * exx + z2 * ezz + z3 * qxx + z3 * qzz;
    const T PRv = q1 * exx + q2 * ezz + q3 * qxx + q3 * qzz;
    oxx[r] = oxx[r] + p.DTE * TXXv;
    ozz[r] = ozz[r] + p.DTE * TZZv;
    opr[r] = opr[r] + p.DTE * PRv;
  }
  // every load above precedes every store (a load may not pass a store
  // to memory it could alias, so interleaving would serialise the rows)
#pragma unroll
  for (int r = 0; r < kRZS; ++r) {
    p.oTXZ[c0 + r * P] = oxz[r]; p.oTXX[c0 + r * P] = oxx[r];
    p.oTZZ[c0 + r * P] = ozz[r]; p.oPRES[c0 + r * P] = opr[r];
  }
}

// velocity: qx and u need 4 <= I <= MX-2 (inh_qx_int.F90:40); qz and w
// (3..MX-2) cover that range
template <class T>
__device__ __forceinline__ bool velocity_fast_rows(const Params<T>& p, int I, int L0) {
  const int I0 = I - (int)(threadIdx.x & 31);
  return L0 >= 2 && L0 + kRZV - 1 <= p.MZ - 2 && I0 >= 4 && I0 + 31 <= p.MX - 2;
}

template <class T, int MODE>
__device__ __forceinline__ void velocity_interior_rows(const Params<T>& p, int I, int L0) {
  const long long P = p.pitch;
  const long long c0 = (long long)L0 * P + (I - p.PMLL);
  const T A = p.A, B = p.B;
  const T* XX = p.TXX + c0;
  const T* ZZ = p.TZZ + c0;
  const T* XZ = p.TXZ + c0;
  const T* PR = p.PRES + c0;
  // xz[k] = TXZ(I, L0-1+k); zz[k], pr[k] = TZZ, PRES(I, L0-2+k)
  T xz[kRZV + 3], zz[kRZV + 3], pr[kRZV + 3];
#pragma unroll
  for (int k = 0; k < kRZV + 3; ++k) {
    xz[k] = __ldg(XZ + (k - 1) * P);
    zz[k] = __ldg(ZZ + (k - 2) * P);
    pr[k] = __ldg(PR + (k - 2) * P);
  }
  // the velocities of all rows; they receive the new values
  T oqx[kRZV], oum[kRZV], oqz[kRZV], owm[kRZV];
#pragma unroll
  for (int r = 0; r < kRZV; ++r) {
    oqx[r] = p.QX[c0 + r * P]; oum[r] = p.UM[c0 + r * P];
    oqz[r] = p.QZ[c0 + r * P]; owm[r] = p.WM[c0 + r * P];
  }
#pragma unroll
  for (int r = 0; r < kRZV; ++r) {
    const long long cell_ = c0 + r * P;
    const int J_ = (MODE == M_TABLE) ? p.JM[cell_] : 0;
    const T* XXr = XX + r * P;
    const T* XZr = XZ + r * P;
    const T* PRr = PR + r * P;
    {
      // inh_qx_int.F90:44-52 and inh_v_uv_int.F90:45-54
      const T E = FDP_C(C_EQX), Cu = FDP_C(C_CU);
      const T R1 = FDP_C(C_R1QX), R2 = FDP_C(C_R2QX), R1u = FDP_C(C_R1U), R3u = FDP_C(C_R3U);
      const T qx0 = oqx[r], u0 = oum[r];
      const T X = A * (__ldg(XXr + 1) - __ldg(XXr - 2) + xz[r + 3] - xz[r])
                + B * (__ldg(XXr) - __ldg(XXr - 1) + xz[r + 2] - xz[r + 1]);
      const T Pp = A * (__ldg(PRr + 1) - __ldg(PRr - 2)) + B * (pr[r + 2] - __ldg(PRr - 1));
      oqx[r] = E * qx0 - R1 * X - R2 * Pp;
      oum[r] = u0 + Cu * qx0 + R1u * X + R3u * Pp;
    }
    {
      // inh_qz_int.F90:45-53 and inh_v_w_int.F90:47-56
      const T E = FDP_C(C_EQZ), Cw = FDP_C(C_CW);
      const T R1 = FDP_C(C_R1QZ), R2 = FDP_C(C_R2QZ), R1w = FDP_C(C_R1W), R3w = FDP_C(C_R3W);
      const T qz0 = oqz[r], w0 = owm[r];
      const T X = A * (zz[r + 3] - zz[r] + __ldg(XZr + 2) - __ldg(XZr - 1))
                + B * (zz[r + 2] - zz[r + 1] + __ldg(XZr + 1) - xz[r + 1]);
      const T Pp = A * (pr[r + 3] - pr[r]) + B * (pr[r + 2] - pr[r + 1]);
      oqz[r] = E * qz0 - R1 * X - R2 * Pp;
      owm[r] = w0 + Cw * qz0 + R1w * X + R3w * Pp;
    }
  }
  // every load above precedes every store (a load may not pass a store
  // to memory it could alias, so interleaving would serialise the rows)
#pragma unroll
  for (int r = 0; r < kRZV; ++r) {
    p.oQX[c0 + r * P] = oqx[r]; p.oUM[c0 + r * P] = oum[r];
    p.oQZ[c0 + r * P] = oqz[r]; p.oWM[c0 + r * P] = owm[r];
  }
}

// ---------------------------------------------------------------------------
// Stencil neighbours are read through a reader: rd(f, I, L) returns input
// field f of the phase (velocities u w qx qz in the stress phase; stresses
// txx tzz txz p in the velocity phase) at cell (I, L).
template <class T> struct GlobalRd {
  const T* f[4];
  long long pitch;
  int PMLL;
  __device__ __forceinline__ T operator()(int k, int I, int L) const {
    return __ldg(f[k] + (long long)L * pitch + (I - PMLL));
  }
};

// The same through the coherent path, for cells whose inputs the running
// kernel itself writes first (the stress-imaging row 1 written at the start
// of a stress phase).
template <class T> struct GlobalRdC {
  const T* f[4];
  long long pitch;
  int PMLL;
  __device__ __forceinline__ T operator()(int k, int I, int L) const {
    return f[k][(long long)L * pitch + (I - PMLL)];
  }
};

// ---------------------------------------------------------------------------
// strain_uw_xx.F90:59-107 / strain_q_xx.F90:54-100 for one cell
template <class T, class R>
__device__ __forceinline__ T strain_xx(const Params<T>& p, const R& rd, int f, T* ML, T* MH, int I, int L) {
  const int TPML = p.TPML;
  if (I <= 1) {
    const int xi = (2 - I) + L * (TPML + 1);
    const int mi = (I - p.PMLL) + L * (TPML + 1);
    const T D = p.CH * (rd(f, I + 1, L) - rd(f, I, L));
    const T m = ML[mi];
    const T e = p.ODA_XL[xi] * (p.ODD_XL[xi] * D + m);
    ML[mi] = p.ODB_XL[xi] * m + p.ODC_XL[xi] * D;
    return e;
  }
  if (I == 2) return p.CH * (rd(f, 3, L) - rd(f, 2, L));
  if (I <= p.MX - 2)
    return p.AH * (rd(f, I + 2, L) - rd(f, I - 1, L)) + p.BH * (rd(f, I + 1, L) - rd(f, I, L));
  if (I == p.MX1) return p.CH * (rd(f, p.MX1 + 1, L) - rd(f, p.MX1, L));
  const int xi = (I - p.MX1) + L * (TPML + 1);
  const int mi = (I - p.MX) + L * (TPML + 1);
  const T D = p.CH * (rd(f, I + 1, L) - rd(f, I, L));
  const T m = MH[mi];
  const T e = p.ODA_XH[xi] * (p.ODD_XH[xi] * D + m);
  MH[mi] = p.ODB_XH[xi] * m + p.ODC_XH[xi] * D;
  return e;
}

// strain_uw_zz.F90:48-60 / strain_q_zz.F90:45-58 (interior and non-imaging row 1)
template <class T, class R>
__device__ __forceinline__ T strain_zz(const Params<T>& p, const R& rd, int f, int I, int L) {
  T e = (p.CH * (rd(f, I, L + 1) - rd(f, I, L)));
  if (I >= 2 && I <= p.MX1) e = p.AH * (rd(f, I, L + 2) - rd(f, I, L - 1)) + p.BC * e;
  return e;
}

// strain_uw_zz_2nd_pml.F90:55-65 / strain_q_zz_2nd_pml.F90:51-64
template <class T, class R>
__device__ __forceinline__ T strain_zz_pml(const Params<T>& p, const R& rd, int f, T* M, int I, int L, int LL) {
  const int zi = (I - p.PMLL) + LL * p.NX;
  const T D = p.CH * (rd(f, I, L + 1) - rd(f, I, L));
  const T m = M[zi];
  const T e = p.ODA_ZH[zi] * (p.ODD_ZH[zi] * D + m);
  M[zi] = p.ODB_ZH[zi] * m + p.ODC_ZH[zi] * D;
  return e;
}

// ---------------------------------------------------------------------------
// Stress update of one cell (I, L): the row routines of hplane_ic_stress,
// hplane_lin_stress, hplane_0/1_stress (non-imaging), hplane_mz1_stress,
// hplane_pml_stress and hplane_pmlzh0_stress restricted to that cell.
//
// Every value the cell reads is loaded first -- the velocity neighbourhood
// unconditionally (the neighbours lie in the arrays' padding where they are
// unused), the PML memory variables and profiles of its region, its
// coefficients and its old stresses -- then the arithmetic runs, then every
// store: a frame cell costs one round trip to memory instead of one per
// strain, whose memory-variable stores would otherwise order the next
// strain's loads behind them.
template <class T, bool SI, int MODE, class R>
__device__ __forceinline__ void stress_cell(const Params<T>& p, const R& rd, int I, int L, int it) {
  const int TPML = p.TPML, MX = p.MX, MX1 = p.MX1;
  const long long cell_ = (long long)L * p.pitch + (I - p.PMLL);
  const int J_ = (MODE == M_TABLE) ? p.JM[cell_] : 0;
  const bool last = (L == p.PMLZH);
  const bool pml = (L >= p.MZ) && !last;
  const bool mz1 = (L == p.MZ - 1);
  const bool r0 = (!SI) && (L == 0);
  const bool r1 = (!SI) && (L == 1);
  const bool do_xz = I >= 2 - TPML && I <= MX + TPML;            // stress_xz.F90:40
  const bool do_nn = !last && I >= 2 - TPML && I <= MX1 + TPML;  // stress_nn.F90:49

  // ---- loads
  // u: column I rows L-2..L+1 and row L columns I-1..I+2; w: row L columns
  // I-2..I+1 and column I rows L-1..L+2; qx: row L columns I-1..I+2; qz:
  // column I rows L-1..L+2
  const T u_m2 = rd(0, I, L - 2), u_m1 = rd(0, I, L - 1), u_0 = rd(0, I, L), u_p1 = rd(0, I, L + 1);
  const T u_xm1 = rd(0, I - 1, L), u_xp1 = rd(0, I + 1, L), u_xp2 = rd(0, I + 2, L);
  const T w_xm2 = rd(1, I - 2, L), w_xm1 = rd(1, I - 1, L), w_0 = rd(1, I, L), w_xp1 = rd(1, I + 1, L);
  const T w_m1 = rd(1, I, L - 1), w_p1 = rd(1, I, L + 1), w_p2 = rd(1, I, L + 2);
  const T x_m1 = rd(2, I - 1, L), x_0 = rd(2, I, L), x_p1 = rd(2, I + 1, L), x_p2 = rd(2, I + 2, L);
  const T z_m1 = rd(3, I, L - 1), z_0 = rd(3, I, L), z_p1 = rd(3, I, L + 1), z_p2 = rd(3, I, L + 2);
  // exz: the z-PML part (strain_uw_xz_2nd_pml.F90) and the x-PML part of
  // the side strips (strain_uw_xz.F90:61-76, 209-223 and the PML rows)
  const bool xz_z = do_xz && !r0 && (pml || last);
  const bool xz_lo = do_xz && !r0 && I <= 2, xz_hi = do_xz && !r0 && I > MX1;
  const int zi = (I - p.PMLL) + (last ? TPML + 1 : L - p.MZ + 1) * p.NX;
  T mz = T(0), za = T(0), zd = T(0), zb = T(0), zc = T(0);
  if (xz_z) { mz = p.PXZH[zi]; za = p.ODA2_ZH[zi]; zd = p.ODD2_ZH[zi]; zb = p.ODB2_ZH[zi]; zc = p.ODC2_ZH[zi]; }
  const int xz_xi = xz_lo ? (3 - I) + L * (TPML + 2) : (I - MX1) + L * (TPML + 2);
  const int xz_mi = xz_lo ? (I - p.PMLL) + L * (TPML + 2) : (I - MX) + L * (TPML + 1);
  T* const xz_m = xz_lo ? p.PZXL : p.PZXH;
  T mx = T(0), xa = T(0), xd = T(0), xb = T(0), xc = T(0);
  if (xz_lo || xz_hi) {
    const T* a_ = xz_lo ? p.ODA2_XL : p.ODA2_XH;
    const T* d_ = xz_lo ? p.ODD2_XL : p.ODD2_XH;
    const T* b_ = xz_lo ? p.ODB2_XL : p.ODB2_XH;
    const T* c_ = xz_lo ? p.ODC2_XL : p.ODC2_XH;
    mx = xz_m[xz_mi]; xa = a_[xz_xi]; xd = d_[xz_xi]; xb = b_[xz_xi]; xc = c_[xz_xi];
  }
  // ezz, qzz in the PML rows and row MZ-1 (strain_*_zz_2nd_pml.F90)
  const bool zz_pml = do_nn && !r0 && (pml || mz1);
  const int zj = (I - p.PMLL) + (mz1 ? 0 : L - p.MZ + 1) * p.NX;
  T me = T(0), mq = T(0), pa = T(0), pd = T(0), pb = T(0), pc = T(0);
  if (zz_pml) { me = p.PZZH[zj]; mq = p.OZZH[zj]; pa = p.ODA_ZH[zj]; pd = p.ODD_ZH[zj]; pb = p.ODB_ZH[zj]; pc = p.ODC_ZH[zj]; }
  // exx, qxx in the side strips (strain_uw_xx.F90:59-107, strain_q_xx.F90:54-100)
  const bool xx_lo = do_nn && I <= 1, xx_hi = do_nn && I >= MX;
  const int xx_xi = xx_lo ? (2 - I) + L * (TPML + 1) : (I - MX1) + L * (TPML + 1);
  const int xx_mi = xx_lo ? (I - p.PMLL) + L * (TPML + 1) : (I - MX) + L * (TPML + 1);
  T* const xx_me = xx_lo ? p.PXXL : p.PXXH;
  T* const xx_mq = xx_lo ? p.OXXL : p.OXXH;
  T ne = T(0), nq = T(0), qa = T(0), qd = T(0), qb = T(0), qc = T(0);
  if (xx_lo || xx_hi) {
    const T* a_ = xx_lo ? p.ODA_XL : p.ODA_XH;
    const T* d_ = xx_lo ? p.ODD_XL : p.ODD_XH;
    const T* b_ = xx_lo ? p.ODB_XL : p.ODB_XH;
    const T* c_ = xx_lo ? p.ODC_XL : p.ODC_XH;
    ne = xx_me[xx_mi]; nq = xx_mq[xx_mi]; qa = a_[xx_xi]; qd = d_[xx_xi]; qb = b_[xx_xi]; qc = c_[xx_xi];
  }
  T cmu = T(0), txz0 = T(0);
  if (do_xz) { cmu = FDP_C(C_MU); txz0 = FDP_F(p.TXZ, I, L); }
  T s1 = T(0), s2 = T(0), s3 = T(0), z1 = T(0), z2 = T(0), z3 = T(0), q1 = T(0), q2 = T(0), q3 = T(0);
  T txx0 = T(0), tzz0 = T(0), pr0 = T(0);
  if (do_nn) {
    s1 = FDP_C(C_SXX1); s2 = FDP_C(C_SXX2); s3 = FDP_C(C_SXX3);
    z1 = FDP_C(C_SZZ1); z2 = FDP_C(C_SZZ2); z3 = FDP_C(C_SZZ3);
    q1 = FDP_C(C_P1); q2 = FDP_C(C_P2); q3 = FDP_C(C_P3);
    txx0 = FDP_F(p.TXX, I, L); tzz0 = FDP_F(p.TZZ, I, L); pr0 = FDP_F(p.PRES, I, L);
  }

  // ---- arithmetic (the reference's expressions and order)
  T exz = T(0), mz_new = T(0), mx_new = T(0);
  if (do_xz) {
    if (r0) {
      exz = T(0);  // hplane_0_stress.F90:58
    } else if (pml || last) {
      // strain_uw_xz_2nd_pml.F90:69-121
      const T DZXA = p.CH * (w_0 - w_xm1);
      const T DXZA = p.CH * (u_0 - u_m1);
      const T zpart = za * (zd * DXZA + mz);
      if (xz_lo || xz_hi) {
        exz = zpart + xa * (xd * DZXA + mx);
        mx_new = xb * mx + xc * DZXA;
      } else {
        exz = zpart + DZXA;
      }
      mz_new = zb * mz + zc * DXZA;
    } else if (xz_lo || xz_hi) {
      // strain_uw_xz.F90:61-76, 209-223 (and strain_uw_xz_1.F90:62-76)
      const T DZXA = p.CH * (w_0 - w_xm1);
      exz = p.CH * (u_0 - u_m1) + xa * (xd * DZXA + mx);
      mx_new = xb * mx + xc * DZXA;
    } else if (r1) {
      // strain_uw_xz_1.F90:79-97 (AFDA_XZ undefined)
      exz = p.AH * (w_xp1 - w_xm2) + p.BH * (w_0 - w_xm1) + p.CH * (u_0 - u_m1);
    } else {
      // strain_uw_xz.F90:78-86
      exz = p.AH * (u_p1 - u_m2 + w_xp1 - w_xm2) + p.BH * (u_0 - u_m1 + w_0 - w_xm1);
    }
  }
  // stress_xz.F90:44-46
  const T TXZv = cmu * exz;
  const T txz_new = txz0 + p.DTE * TXZv;

  T txx_new = T(0), tzz_new = T(0), pr_new = T(0), me_new = T(0), mq_new = T(0), ne_new = T(0), nq_new = T(0);
  if (do_nn) {
    T ezz, qzz;
    if (r0) {
      ezz = (p.CH * (w_p1 - w_0));  // strain_uw_zz_0.F90:45-49
      qzz = (p.CH * (z_p1 - z_0));  // strain_q_zz_0.F90:40-44
    } else if (pml || mz1) {
      // strain_uw_zz_2nd_pml.F90:55-65 / strain_q_zz_2nd_pml.F90:51-64
      const T De = p.CH * (w_p1 - w_0);
      ezz = pa * (pd * De + me);
      me_new = pb * me + pc * De;
      const T Dq = p.CH * (z_p1 - z_0);
      qzz = pa * (pd * Dq + mq);
      mq_new = pb * mq + pc * Dq;
    } else {
      // strain_uw_zz.F90:48-60 / strain_q_zz.F90:45-58
      ezz = (p.CH * (w_p1 - w_0));
      if (I >= 2 && I <= MX1) ezz = p.AH * (w_p2 - w_m1) + p.BC * ezz;
      qzz = (p.CH * (z_p1 - z_0));
      if (I >= 2 && I <= MX1) qzz = p.AH * (z_p2 - z_m1) + p.BC * qzz;
    }
    // strain_uw_xx.F90:59-107 / strain_q_xx.F90:54-100
    T exx, qxx;
    if (xx_lo || xx_hi) {
      const T De = p.CH * (u_xp1 - u_0);
      exx = qa * (qd * De + ne);
      ne_new = qb * ne + qc * De;
      const T Dq = p.CH * (x_p1 - x_0);
      qxx = qa * (qd * Dq + nq);
      nq_new = qb * nq + qc * Dq;
    } else if (I == 2 || I == MX1) {
      exx = p.CH * (u_xp1 - u_0);
      qxx = p.CH * (x_p1 - x_0);
    } else {
      exx = p.AH * (u_xp2 - u_xm1) + p.BH * (u_xp1 - u_0);
      qxx = p.AH * (x_p2 - x_m1) + p.BH * (x_p1 - x_0);
    }
    // stress_nn.F90:53-59
    const T TXXv = s1 * exx + s2 * ezz + s3 * qxx + s3 * qzz;
    const T TZZv = z1 * exx + z2 * ezz + z3 * qxx + z3 * qzz;
    const T PRv = q1 * exx + q2 * ezz + q3 * qxx + q3 * qzz;
    if (L == p.LIN_Z && I == p.LIN_X) {
      // stress_lin_nn.F90:58-63; SOURSP/SOURFP are the previous level's values
      const T SOURS = p.STF[2 * (it - 1)], SOURF = p.STF[2 * (it - 1) + 1];
      const T SOURSP = it > 1 ? p.STF[2 * (it - 2)] : T(0);
      const T SOURFP = it > 1 ? p.STF[2 * (it - 2) + 1] : T(0);
      txx_new = txx0 + p.DTE * (TXXv - ((SOURS - SOURSP) / p.DT));
      tzz_new = tzz0 + p.DTE * (TZZv - ((SOURS - SOURSP) / p.DT));
      pr_new = pr0 + p.DTE * (PRv + ((SOURF - SOURFP) / p.DT));
    } else {
      txx_new = txx0 + p.DTE * TXXv;
      tzz_new = tzz0 + p.DTE * TZZv;
      pr_new = pr0 + p.DTE * PRv;
    }
  }

  // ---- stores
  if (do_xz) {
    if (xz_z) p.PXZH[zi] = mz_new;
    if (xz_lo || xz_hi) xz_m[xz_mi] = mx_new;
    FDP_F(p.oTXZ, I, L) = txz_new;
  }
  if (do_nn) {
    if (zz_pml) { p.PZZH[zj] = me_new; p.OZZH[zj] = mq_new; }
    if (xx_lo || xx_hi) { xx_me[xx_mi] = ne_new; xx_mq[xx_mi] = nq_new; }
    FDP_F(p.oTXX, I, L) = txx_new;
    FDP_F(p.oTZZ, I, L) = tzz_new;
    FDP_F(p.oPRES, I, L) = pr_new;
  }
}

// One thread per kRZS cells of a column; a unit of kBX x kBZ threads covers
// kBX columns (from I0, none at or beyond I1 <= PMLXH+1) and kBZ*kRZS rows.
// Unit rows tile the grid from row 0 down, so unit row 0 holds rows 2..4
// that the stress-imaging mirror rows 0 and 1 copy.  k_stress runs one unit
// per block, the frame and batched kernels the units of their lists.
// stress_unit's cells of thread (tx, ty) of the unit, without the
// stress-imaging mirror rows.
template <class T, bool SI, int MODE, bool COH = false>
__device__ __forceinline__ void stress_unit_cells(const Params<T>& p, int I0, int I1, int by, int it_off, int tx,
                                                  int ty) {
  const int I = I0 + tx;
  const int L0 = (by * kBZ + ty) * kRZS;  // rows L0 .. L0+kRZS-1
  const bool core = p.cs_x1 > p.cs_x0;  // the core kernel updates the core cells
  if (!COH && !core && I1 > p.PMLXH && stress_fast_rows(p, I, L0)) {
    stress_interior_rows<T, MODE>(p, I, L0);
  } else if (I < I1) {
    const int it = *p.it_base + it_off;
    using Rd = typename std::conditional<COH, GlobalRdC<T>, GlobalRd<T>>::type;
    const Rd rd{{p.UM, p.WM, p.QX, p.QZ}, p.pitch, p.PMLL};
    const bool incol = I >= p.cs_x0 && I < p.cs_x1;
#pragma unroll 1
    for (int L = L0; L < L0 + kRZS; ++L)
      if (L <= p.PMLZH && (!SI || L >= 2) &&
          !(incol && L >= p.cs_z0 && L < p.cs_z1 && (p.cs_src || L != p.LIN_Z)))
        stress_cell<T, SI, MODE>(p, rd, I, L, it);
  }
}

// The stress-imaging mirror rows 0 and 1 of column I from the new rows
// 2..4 (hplane_0_stress.F90:49-53 and hplane_1_stress.F90:45-53).
template <class T>
__device__ __forceinline__ void stress_mirror(const Params<T>& p, int I) {
  FDP_F(p.oTXZ, I, 0) = -FDP_F(p.oTXZ, I, 4);
  FDP_F(p.oTZZ, I, 0) = -FDP_F(p.oTZZ, I, 3);
  FDP_F(p.oPRES, I, 0) = -FDP_F(p.oPRES, I, 3);
  FDP_F(p.oTXZ, I, 1) = -FDP_F(p.oTXZ, I, 3);
  FDP_F(p.oTZZ, I, 1) = -FDP_F(p.oTZZ, I, 2);
  FDP_F(p.oPRES, I, 1) = -FDP_F(p.oPRES, I, 2);
  FDP_F(p.oTXZ, I, 2) = T(0);
}

template <class T, bool SI, int MODE, bool COH = false>
__device__ __forceinline__ void stress_unit(const Params<T>& p, int I0, int I1, int by, int it_off) {
  stress_unit_cells<T, SI, MODE, COH>(p, I0, I1, by, it_off, (int)threadIdx.x, (int)threadIdx.y);
  if (SI && by == 0) {
    __syncthreads();  // rows 2..4 of this unit are final
    if (I0 + (int)threadIdx.x < I1 && threadIdx.y == 0) stress_mirror(p, I0 + (int)threadIdx.x);
  }
}

template <class T, bool SI, int MODE>
__global__ void __launch_bounds__(kBX * kBZ) k_stress(const __grid_constant__ Params<T> p, int it_off) {
  stress_unit<T, SI, MODE>(p, p.PMLL + (int)blockIdx.x * kBX, p.PMLXH + 1, (int)blockIdx.y, it_off);
}

// ---------------------------------------------------------------------------
// Velocity update of one cell (I, L), L < PMLZH: hplane_ic_velocity,
// hplane_pml_velocity and, without stress imaging, hplane_0/1_velocity.
// The old q at the cell stands in for QXP/QZP: STO_QXP/STO_QZP copy q right
// after its update over exactly the columns and rows where u and w read the
// copy (sto_qxp.F90:24, sto_qzp.F90:24), so QXP(I,L) always equals the q of
// the previous level at that cell.
template <class T, bool SI, int MODE, class R>
__device__ __forceinline__ void velocity_cell(const Params<T>& p, const R& rd, int I, int L) {
  const int TPML = p.TPML, MX = p.MX, MX1 = p.MX1;
  const long long cell_ = (long long)L * p.pitch + (I - p.PMLL);
  const int J_ = (MODE == M_TABLE) ? p.JM[cell_] : 0;
  const bool pml = (L >= p.MZ - 1);
  const T A = p.A, B = p.B;

  // ---------------- qx and u: I = 3-TPML .. MX-1+TPML
  if (I >= 3 - TPML && I <= MX1 + TPML) {
    const T E = FDP_C(C_EQX), Cu = FDP_C(C_CU);
    const T R1 = FDP_C(C_R1QX), R2 = FDP_C(C_R2QX), R1u = FDP_C(C_R1U), R3u = FDP_C(C_R3U);
    const T qx0 = FDP_F(p.QX, I, L);
    const T u0 = FDP_F(p.UM, I, L);
    T qx, u;
    if (pml) {
      // inh_qx_int_2nd_pml.F90 / inh_v_u_int_2nd_pml.F90
      const int LL = L - p.MZ + 1;
      const int zi = (I - p.PMLL) + LL * p.NX;
      const T DXXXA = rd(0, I, L) - rd(0, I - 1, L);
      const T DXZZA = rd(2, I, L + 1) - rd(2, I, L);
      const T PXXXA = rd(3, I, L) - rd(3, I - 1, L);
      const T za = p.ODA_ZH[zi], zd = p.ODD_ZH[zi], zb = p.ODB_ZH[zi], zc = p.ODC_ZH[zi];
      const T gz = p.GXZH[zi], rz = p.RXZH[zi];
      if (I <= 3 || I >= MX1) {
        int xi, mi;
        const T *xa_, *xd_, *xb_, *xc_;
        T *G, *H, *Rm, *S;
        if (I <= 3) {
          xi = (3 - I) + L * (TPML + 2); mi = (I - p.PMLL) + L * (TPML + 3);
          xa_ = p.ODA2_XL; xd_ = p.ODD2_XL; xb_ = p.ODB2_XL; xc_ = p.ODC2_XL;
          G = p.GXXL; H = p.HXXL; Rm = p.RXXL; S = p.SXXL;
        } else {
          xi = (I - MX1) + L * (TPML + 2); mi = (I - (MX - 1)) + L * (TPML + 2);
          xa_ = p.ODA2_XH; xd_ = p.ODD2_XH; xb_ = p.ODB2_XH; xc_ = p.ODC2_XH;
          G = p.GXXH; H = p.HXXH; Rm = p.RXXH; S = p.SXXH;
        }
        const T xa = xa_[xi], xd = xd_[xi], xb = xb_[xi], xc = xc_[xi];
        const T g = G[mi], h = H[mi], r = Rm[mi], s = S[mi];
        qx = E * qx0 - R1 * (xa * (xd * DXXXA + g)) - R1 * (za * (zd * DXZZA + gz)) - R2 * (xa * (xd * PXXXA + h));
        u = u0 + Cu * qx0 + R1u * (xa * (xd * DXXXA + r) + za * (zd * DXZZA + rz)) + R3u * (xa * (xd * PXXXA + s));
        G[mi] = xb * g + xc * DXXXA;
        H[mi] = xb * h + xc * PXXXA;
        Rm[mi] = xb * r + xc * DXXXA;
        S[mi] = xb * s + xc * PXXXA;
      } else {
        qx = E * qx0 - R1 * (za * (zd * DXZZA + gz) + DXXXA) - R2 * (rd(3, I, L) - rd(3, I - 1, L));
        u = u0 + Cu * qx0 + R1u * (DXXXA + za * (zd * DXZZA + rz)) + R3u * PXXXA;
      }
      p.GXZH[zi] = zb * gz + zc * DXZZA;
      p.RXZH[zi] = zb * rz + zc * DXZZA;
    } else if (SI || L >= 1) {
      // interior rows, and row 1 without stress imaging (the same routines)
      if (I <= 3 || I >= MX1) {
        // inh_qx_2nd.F90 / inh_v_u_2nd.F90
        int xi, mi;
        const T *xa_, *xd_, *xb_, *xc_;
        T *G, *H, *Rm, *S;
        if (I <= 3) {
          xi = (3 - I) + L * (TPML + 2); mi = (I - p.PMLL) + L * (TPML + 3);
          xa_ = p.ODA2_XL; xd_ = p.ODD2_XL; xb_ = p.ODB2_XL; xc_ = p.ODC2_XL;
          G = p.GXXL; H = p.HXXL; Rm = p.RXXL; S = p.SXXL;
        } else {
          xi = (I - MX1) + L * (TPML + 2); mi = (I - (MX - 1)) + L * (TPML + 2);
          xa_ = p.ODA2_XH; xd_ = p.ODD2_XH; xb_ = p.ODB2_XH; xc_ = p.ODC2_XH;
          G = p.GXXH; H = p.HXXH; Rm = p.RXXH; S = p.SXXH;
        }
        const T DXXXA = rd(0, I, L) - rd(0, I - 1, L);
        const T PXXXA = rd(3, I, L) - rd(3, I - 1, L);
        const T txz1 = rd(2, I, L + 1), txz0 = rd(2, I, L);
        const T xa = xa_[xi], xd = xd_[xi], xb = xb_[xi], xc = xc_[xi];
        const T g = G[mi], h = H[mi], r = Rm[mi], s = S[mi];
        qx = E * qx0 - R1 * (xa * (xd * DXXXA + g) + txz1 - txz0) - R2 * (xa * (xd * PXXXA + h));
        u = u0 + Cu * qx0 + R1u * (xa * (xd * DXXXA + r) + txz1 - txz0) + R3u * (xa * (xd * PXXXA + s));
        G[mi] = xb * g + xc * DXXXA;
        H[mi] = xb * h + xc * PXXXA;
        Rm[mi] = xb * r + xc * DXXXA;
        S[mi] = xb * s + xc * PXXXA;
      } else {
        // inh_qx_int.F90:40-54 / inh_v_uv_int.F90:41-56
        const T X = A * (rd(0, I + 1, L) - rd(0, I - 2, L) + rd(2, I, L + 2) - rd(2, I, L - 1))
                  + B * (rd(0, I, L) - rd(0, I - 1, L) + rd(2, I, L + 1) - rd(2, I, L));
        const T P = A * (rd(3, I + 1, L) - rd(3, I - 2, L)) + B * (rd(3, I, L) - rd(3, I - 1, L));
        qx = E * qx0 - R1 * X - R2 * P;
        u = u0 + Cu * qx0 + R1u * X + R3u * P;
      }
    } else {
      // row 0 without stress imaging: inh_qx_int_0.F90, inh_v_uv_int_0.F90,
      // inh_qx_2nd_0.F90, inh_v_u_2nd_0.F90
      if (I <= 3 || I >= MX1) {
        int xi, mi;
        const T *xa_, *xd_, *xb_, *xc_;
        T *G, *H, *Rm, *S;
        if (I <= 3) {
          xi = (3 - I); mi = (I - p.PMLL);
          xa_ = p.ODA2_XL; xd_ = p.ODD2_XL; xb_ = p.ODB2_XL; xc_ = p.ODC2_XL;
          G = p.GXXL; H = p.HXXL; Rm = p.RXXL; S = p.SXXL;
        } else {
          xi = (I - MX1); mi = (I - (MX - 1));
          xa_ = p.ODA2_XH; xd_ = p.ODD2_XH; xb_ = p.ODB2_XH; xc_ = p.ODC2_XH;
          G = p.GXXH; H = p.HXXH; Rm = p.RXXH; S = p.SXXH;
        }
        const T DXXXA = rd(0, I, 0) - rd(0, I - 1, 0);
        const T PXXXA = rd(3, I, 0) - rd(3, I - 1, 0);
        const T txz1 = rd(2, I, 1);
        const T xa = xa_[xi], xd = xd_[xi], xb = xb_[xi], xc = xc_[xi];
        const T g = G[mi], h = H[mi], r = Rm[mi], s = S[mi];
        qx = E * qx0 - R1 * (xa * (xd * DXXXA + g) + txz1) - R2 * (xa * (xd * PXXXA + h));
        u = u0 + Cu * qx0 + R1u * (xa * (xd * DXXXA + r) + txz1) + R3u * (xa * (xd * PXXXA + s));
        G[mi] = xb * g + xc * DXXXA;
        H[mi] = xb * h + xc * PXXXA;
        Rm[mi] = xb * r + xc * DXXXA;
        S[mi] = xb * s + xc * PXXXA;
      } else {
        const T X = A * (rd(0, I + 1, 0) - rd(0, I - 2, 0)) + B * (rd(0, I, 0) - rd(0, I - 1, 0))
                  + T(17) / T(24) * rd(2, I, 1) + T(3) / T(8) * rd(2, I, 2)
                  - T(5) / T(24) * rd(2, I, 3) + T(1) / T(24) * rd(2, I, 4);
        const T P = A * (rd(3, I + 1, 0) - rd(3, I - 2, 0)) + B * (rd(3, I, 0) - rd(3, I - 1, 0));
        qx = E * qx0 - R1 * X - R2 * P;
        u = u0 + Cu * qx0 + R1u * X + R3u * P;
      }
    }
    FDP_F(p.oQX, I, L) = qx;
    FDP_F(p.oUM, I, L) = u;
  }

  // ---------------- qz and w: I = 2-TPML .. MX-1+TPML
  if (I >= 2 - TPML && I <= MX1 + TPML) {
    const T E = FDP_C(C_EQZ), Cw = FDP_C(C_CW);
    const T R1 = FDP_C(C_R1QZ), R2 = FDP_C(C_R2QZ), R1w = FDP_C(C_R1W), R3w = FDP_C(C_R3W);
    const T qz0 = FDP_F(p.QZ, I, L);
    const T w0 = FDP_F(p.WM, I, L);
    T qz, w;
    if (pml) {
      // inh_qz_int_2nd_pml.F90 / inh_v_w_int_2nd_pml.F90
      const int LL = L - p.MZ + 1;
      const int zi = (I - p.PMLL) + LL * p.NX;
      const T DXZXA = rd(2, I + 1, L) - rd(2, I, L);
      const T DZZZA = rd(1, I, L) - rd(1, I, L - 1);
      const T PZZZA = rd(3, I, L) - rd(3, I, L - 1);
      const T za = p.ODA2_ZH[zi], zd = p.ODD2_ZH[zi], zb = p.ODB2_ZH[zi], zc = p.ODC2_ZH[zi];
      const T gz = p.GZZH[zi], hz = p.HZZH[zi], rz = p.RZZH[zi], sz = p.SZZH[zi];
      if (I <= 2 || I >= MX1) {
        int xi, mi;
        const T *xa_, *xd_, *xb_, *xc_;
        T *G, *Rm;
        if (I <= 2) {
          xi = (2 - I) + L * (TPML + 1); mi = (I - p.PMLL) + L * (TPML + 2);
          xa_ = p.ODA_XL; xd_ = p.ODD_XL; xb_ = p.ODB_XL; xc_ = p.ODC_XL; G = p.GZXL; Rm = p.RZXL;
        } else {
          xi = (I - MX1) + L * (TPML + 1); mi = (I - (MX - 1)) + L * (TPML + 2);
          xa_ = p.ODA_XH; xd_ = p.ODD_XH; xb_ = p.ODB_XH; xc_ = p.ODC_XH; G = p.GZXH; Rm = p.RZXH;
        }
        const T xa = xa_[xi], xd = xd_[xi], xb = xb_[xi], xc = xc_[xi];
        const T g = G[mi], r = Rm[mi];
        qz = E * qz0 - R1 * (za * (zd * DZZZA + gz)) - R1 * (xa * (xd * DXZXA + g)) - R2 * (za * (zd * PZZZA + hz));
        w = w0 + Cw * qz0 + R1w * (za * (zd * DZZZA + rz) + xa * (xd * DXZXA + r)) + R3w * (za * (zd * PZZZA + sz));
        G[mi] = xb * g + xc * DXZXA;
        Rm[mi] = xb * r + xc * DXZXA;
      } else {
        qz = E * qz0 - R1 * (za * (zd * DZZZA + gz) + DXZXA) - R2 * (za * (zd * PZZZA + hz));
        w = w0 + Cw * qz0 + R1w * (za * (zd * DZZZA + rz) + DXZXA) + R3w * (za * (zd * PZZZA + sz));
      }
      p.GZZH[zi] = zb * gz + zc * DZZZA;
      p.HZZH[zi] = zb * hz + zc * PZZZA;
      p.RZZH[zi] = zb * rz + zc * DZZZA;
      p.SZZH[zi] = zb * sz + zc * PZZZA;
    } else if (SI || L >= 1) {
      if (I <= 2 || I >= MX1) {
        // inh_qz_2nd.F90 / inh_v_w_2nd.F90 (also row 1 without stress imaging)
        int xi, mi;
        const T *xa_, *xd_, *xb_, *xc_;
        T *G, *Rm;
        if (I <= 2) {
          xi = (2 - I) + L * (TPML + 1); mi = (I - p.PMLL) + L * (TPML + 2);
          xa_ = p.ODA_XL; xd_ = p.ODD_XL; xb_ = p.ODB_XL; xc_ = p.ODC_XL; G = p.GZXL; Rm = p.RZXL;
        } else {
          xi = (I - MX1) + L * (TPML + 1); mi = (I - (MX - 1)) + L * (TPML + 2);
          xa_ = p.ODA_XH; xd_ = p.ODD_XH; xb_ = p.ODB_XH; xc_ = p.ODC_XH; G = p.GZXH; Rm = p.RZXH;
        }
        const T DXZXA = rd(2, I + 1, L) - rd(2, I, L);
        const T dzz = rd(1, I, L) - rd(1, I, L - 1);
        const T dp = rd(3, I, L) - rd(3, I, L - 1);
        const T xa = xa_[xi], xd = xd_[xi], xb = xb_[xi], xc = xc_[xi];
        const T g = G[mi], r = Rm[mi];
        qz = E * qz0 - R1 * (dzz + xa * (xd * DXZXA + g)) - R2 * dp;
        w = w0 + Cw * qz0 + R1w * (dzz + xa * (xd * DXZXA + r)) + R3w * dp;
        G[mi] = xb * g + xc * DXZXA;
        Rm[mi] = xb * r + xc * DXZXA;
      } else if (SI || L >= 2) {
        // inh_qz_int.F90:41-55 / inh_v_w_int.F90:43-58
        const T X = A * (rd(1, I, L + 1) - rd(1, I, L - 2) + rd(2, I + 2, L) - rd(2, I - 1, L))
                  + B * (rd(1, I, L) - rd(1, I, L - 1) + rd(2, I + 1, L) - rd(2, I, L));
        const T P = A * (rd(3, I, L + 1) - rd(3, I, L - 2)) + B * (rd(3, I, L) - rd(3, I, L - 1));
        qz = E * qz0 - R1 * X - R2 * P;
        w = w0 + Cw * qz0 + R1w * X + R3w * P;
      } else {
        // row 1 without stress imaging: inh_v_qz_int_1.F90 / inh_v_w_int_1.F90
        const T X = A * (rd(2, I + 2, 1) - rd(2, I - 1, 1)) + B * (rd(2, I + 1, 1) - rd(2, I, 1))
                  - T(31) / T(24) * rd(1, I, 0) + T(29) / T(24) * rd(1, I, 1)
                  - T(3) / T(40) * rd(1, I, 2) + T(1) / T(168) * rd(1, I, 3);
        const T P = -T(31) / T(24) * rd(3, I, 0) + T(29) / T(24) * rd(3, I, 1)
                  - T(3) / T(40) * rd(3, I, 2) + T(1) / T(168) * rd(3, I, 3);
        qz = E * qz0 - R1 * X - R2 * P;
        w = w0 + Cw * qz0 + R1w * X + R3w * P;
      }
    } else {
      // row 0 without stress imaging: inh_qz_int_0.F90, inh_v_w_int_0.F90,
      // inh_qz_2nd_0.F90, inh_v_w_2nd_0.F90
      T X, P;
      if (I <= 2 || I >= MX1) {
        X = T(3) * rd(1, I, 0) - T(1) / T(3) * rd(1, I, 1);
        P = T(3) * rd(3, I, 0) - T(1) / T(3) * rd(3, I, 1);
      } else {
        X = T(35) / T(8) * rd(1, I, 0) - T(35) / T(24) * rd(1, I, 1)
          + T(21) / T(40) * rd(1, I, 2) - T(5) / T(56) * rd(1, I, 3);
        P = T(35) / T(8) * rd(3, I, 0) - T(35) / T(24) * rd(3, I, 1)
          + T(21) / T(40) * rd(3, I, 2) - T(5) / T(56) * rd(3, I, 3);
      }
      qz = E * qz0 - R1 * X - R2 * P;
      w = w0 + Cw * qz0 + R1w * X + R3w * P;
    }
    FDP_F(p.oQZ, I, L) = qz;
    FDP_F(p.oWM, I, L) = w;
  }
}

// One thread per kRZV cells of a column; units of kBX x kBZ threads tile
// the grid from row PMLZH up, so the thread holding the bottom row also
// holds rows PMLZH-1 and PMLZH-2, whose new values and pre-phase values (the
// history SZ of time_loop.F90:133-155) the bottom row needs.  The pre-phase
// values wait in the thread's own slots of shared memory while it updates
// those rows.
template <class T, bool SI, int MODE>
__device__ __forceinline__ void velocity_unit(const Params<T>& p, int I0, int I1, int by) {
  static_assert(kRZV >= 3, "the bottom row needs two rows above it in the same thread");
  __shared__ T old[3][4][kBX];  // pre-phase values of rows PMLZH-k, k = 0..2
  const int I = I0 + (int)threadIdx.x;
  const int L1 = p.PMLZH - (int)(by * kBZ + (kBZ - 1 - threadIdx.y)) * kRZV;  // last row
  const int L0 = L1 - kRZV + 1;                                                         // first row
  const bool inx = I < I1;
  const bool me = inx && L1 == p.PMLZH;  // this thread updates the bottom row
  const int tx = threadIdx.x;
  if (me) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      old[k][0][tx] = FDP_F(p.UM, I, L1 - k); old[k][1][tx] = FDP_F(p.WM, I, L1 - k);
      old[k][2][tx] = FDP_F(p.QX, I, L1 - k); old[k][3][tx] = FDP_F(p.QZ, I, L1 - k);
    }
  }
  const bool core = p.cv_x1 > p.cv_x0;  // the core kernel updates the core cells
  if (!core && I1 > p.PMLXH && velocity_fast_rows(p, I, L0)) {
    velocity_interior_rows<T, MODE>(p, I, L0);
  } else if (inx) {
    const GlobalRd<T> rd{{p.TXX, p.TZZ, p.TXZ, p.PRES}, p.pitch, p.PMLL};
    const bool incol = I >= p.cv_x0 && I < p.cv_x1;
#pragma unroll 1
    for (int L = L0; L <= L1; ++L)
      if (L >= (SI ? 2 : 0) && L < p.PMLZH && !(incol && L >= p.cv_z0 && L < p.cv_z1))
        velocity_cell<T, SI, MODE>(p, rd, I, L);
  }
  if (me) {
    // hplane_pmlzh0_velocity.F90:34-63
    const int LST = p.PMLZH;
    const int x = I - p.PMLL;
    T* const f[4] = {p.oUM, p.oWM, p.oQX, p.oQZ};  // this phase's new values
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const T* ab = p.AB + ((c == 0 || c == 2) ? 8 : 0);  // ABH for u, qx; ABW for w, qz
      T* hist = p.HIST + (long long)c * 3 * p.NX;
      const T sp0 = hist[x], sp1 = hist[p.NX + x], sp2 = hist[2 * p.NX + x];
      const T v = ab[0] * FDP_F(f[c], I, LST - 1) + ab[1] * FDP_F(f[c], I, LST - 2)
                + ab[2] * old[0][c][tx] + ab[3] * old[1][c][tx] + ab[4] * old[2][c][tx]
                + ab[5] * sp0 + ab[6] * sp1 + ab[7] * sp2;
      FDP_F(f[c], I, LST) = v;
      hist[x] = old[0][c][tx];
      hist[p.NX + x] = old[1][c][tx];
      hist[2 * p.NX + x] = old[2][c][tx];
    }
  }
}

template <class T, bool SI, int MODE>
__global__ void FDP_VELOCITY_BOUNDS(T) k_velocity(const __grid_constant__ Params<T> p, int it_off) {
  (void)it_off;
  velocity_unit<T, SI, MODE>(p, p.PMLL + (int)blockIdx.x * kBX, p.PMLXH + 1, (int)blockIdx.y);
}

// ---------------------------------------------------------------------------
// Frame and core.  With a core rectangle set, each phase is two launches:
// the frame kernels run the unit code over the listed units (those holding
// any cell outside the core), skipping core cells; the core kernels update
// the core, four consecutive cells of a row per thread with 16-byte loads
// and stores.  The core holds only interior cells of the phase (4th-order
// stencils everywhere, no source row), so the core kernels are the interior
// branches of stress_cell / velocity_cell, same expressions in the same
// order, for four cells at a time.
// A frame unit: columns [x, y) (at most kBX), unit row z.  Resident CTAs
// per SM the register allocation aims for (FP32; two in FP64): the cell
// code keeps all of a cell's inputs in registers at once.
#ifndef FDP_STRESS_FRAME_MIN_BLOCKS
#define FDP_STRESS_FRAME_MIN_BLOCKS 3
#endif
template <class T, bool SI>
__device__ __forceinline__ void edge_thread(const Params<T>& p, int g, int it_off);
template <class T>
__device__ __forceinline__ void stress_sample_thread(const Params<T>& p, int g, int it_off);

// Blocks 0..n-1 run the n frame units.  With edge_prev set, the kernel also
// finishes the previous level: the top units first write the
// stress-imaging row 1 of their columns from rows 2 and 3 (which the
// previous velocity phase left final, and which this phase's stresses at
// rows 2 and 3 read), and blocks n.. take the previous level's velocity
// samples of the receivers (velocities stay unchanged through a stress
// phase; row-1 samples are recomputed, not read) and, with edge_prev = 2,
// its stress samples too (when the stresses this kernel reads are the
// previous level's, the new ones going to other arrays).
template <class T, bool SI, int MODE>
__global__ void __launch_bounds__(kBX * kBZ, sizeof(T) == 4 ? FDP_STRESS_FRAME_MIN_BLOCKS : 2) k_stress_frame(const __grid_constant__ Params<T> p,
                                                            const int4* __restrict__ units, int n, int it_off,
                                                            int edge_prev) {
  const int b = (int)blockIdx.x;
  const int tid = (int)(threadIdx.y * kBX + threadIdx.x);
  if (b >= n) {
    edge_thread<T, SI>(p, (SI ? p.NX : 0) + (b - n) * kBX * kBZ + tid, it_off - 1);
    if (edge_prev == 2) stress_sample_thread<T>(p, (b - n) * kBX * kBZ + tid, it_off - 1);
    return;
  }
  const int4 u = units[b];
  if (SI && edge_prev && u.z == 0) {
    if (threadIdx.y == 0 && u.x + (int)threadIdx.x < u.y) edge_thread<T, SI>(p, u.x + (int)threadIdx.x - p.PMLL, it_off - 1);
    __syncthreads();  // row 1 of these columns is final before rows 2 and 3 read it
    stress_unit<T, SI, MODE, true>(p, u.x, u.y, u.z, it_off);
  } else {
    stress_unit<T, SI, MODE>(p, u.x, u.y, u.z, it_off);
  }
}

// Velocity frame cells up to row PMLZH-3, one row per thread: columns
// [I0, I1), rows L0 .. L0+kBZ-1.
template <class T, bool SI, int MODE>
__device__ __forceinline__ void velocity_row_unit(const Params<T>& p, int I0, int I1, int L0, int tx, int ty) {
  const int I = I0 + tx;
  const int L = L0 + ty;
  const bool incore = I >= p.cv_x0 && I < p.cv_x1 && L >= p.cv_z0 && L < p.cv_z1;
  if (I < I1 && L <= p.PMLZH - 3 && L >= (SI ? 2 : 0) && !incore) {
    const GlobalRd<T> rd{{p.TXX, p.TZZ, p.TXZ, p.PRES}, p.pitch, p.PMLL};
    velocity_cell<T, SI, MODE>(p, rd, I, L);
  }
}

// The bottom three rows of columns [I0, I1) (at most kBX*kBZ), one column
// per thread: rows PMLZH-2 and PMLZH-1, then the bottom row from their new
// and pre-phase values and the history (time_loop.F90:133-155,
// hplane_pmlzh0_velocity.F90:34-63).
template <class T, bool SI, int MODE>
__device__ __forceinline__ void velocity_bottom_unit(const Params<T>& p, int I0, int I1, int t) {
  const int I = I0 + t;
  if (I >= I1) return;
  const int LST = p.PMLZH;
  T old[3][4];  // pre-phase values of rows PMLZH-k of u, w, qx, qz
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    old[k][0] = FDP_F(p.UM, I, LST - k); old[k][1] = FDP_F(p.WM, I, LST - k);
    old[k][2] = FDP_F(p.QX, I, LST - k); old[k][3] = FDP_F(p.QZ, I, LST - k);
  }
  const GlobalRd<T> rd{{p.TXX, p.TZZ, p.TXZ, p.PRES}, p.pitch, p.PMLL};
  const bool incol = I >= p.cv_x0 && I < p.cv_x1;
  for (int L = LST - 2; L < LST; ++L)
    if (L >= (SI ? 2 : 0) && !(incol && L >= p.cv_z0 && L < p.cv_z1)) velocity_cell<T, SI, MODE>(p, rd, I, L);
  const int x = I - p.PMLL;
  T* const f[4] = {p.oUM, p.oWM, p.oQX, p.oQZ};  // this phase's new values
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    const T* ab = p.AB + ((c == 0 || c == 2) ? 8 : 0);  // ABH for u, qx; ABW for w, qz
    T* hist = p.HIST + (long long)c * 3 * p.NX;
    const T sp0 = hist[x], sp1 = hist[p.NX + x], sp2 = hist[2 * p.NX + x];
    const T v = ab[0] * FDP_F(f[c], I, LST - 1) + ab[1] * FDP_F(f[c], I, LST - 2)
              + ab[2] * old[0][c] + ab[3] * old[1][c] + ab[4] * old[2][c]
              + ab[5] * sp0 + ab[6] * sp1 + ab[7] * sp2;
    FDP_F(f[c], I, LST) = v;
    hist[x] = old[0][c];
    hist[p.NX + x] = old[1][c];
    hist[2 * p.NX + x] = old[2][c];
  }
}

// A velocity frame unit: (first column, end column, first row, 1) one row
// per thread up to row PMLZH-3, or (first column, end column, 0, 2) the
// bottom three rows.
template <class T, bool SI, int MODE>
__device__ __forceinline__ void velocity_frame_unit(const Params<T>& p, const int4 u) {
  if (u.w == 2) velocity_bottom_unit<T, SI, MODE>(p, u.x, u.y, (int)(threadIdx.y * kBX + threadIdx.x));
  else velocity_row_unit<T, SI, MODE>(p, u.x, u.y, u.z, (int)threadIdx.x, (int)threadIdx.y);
}

// Blocks 0..n-1 run the n frame units; blocks n.. take this level's
// stress samples of the receivers (the velocity phase leaves the stresses
// alone).
template <class T, bool SI, int MODE>
__global__ void __launch_bounds__(kBX * kBZ, sizeof(T) == 4 ? 4 : 2) k_velocity_frame(const __grid_constant__ Params<T> p,
                                                              const int4* __restrict__ units, int n, int it_off) {
  const int b = (int)blockIdx.x;
  if (b >= n) {
    stress_sample_thread<T>(p, (b - n) * kBX * kBZ + (int)(threadIdx.y * kBX + threadIdx.x), it_off);
    return;
  }
  velocity_frame_unit<T, SI, MODE>(p, units[b]);
}

template <class T> struct V4 { T v[4]; };

// four consecutive values at a 16-byte-aligned address, read-only path
__device__ __forceinline__ V4<float> ld4(const float* a) {
  const float4 x = __ldg(reinterpret_cast<const float4*>(a));
  return {{x.x, x.y, x.z, x.w}};
}
__device__ __forceinline__ V4<double> ld4(const double* a) {
  const double2 x = __ldg(reinterpret_cast<const double2*>(a)), y = __ldg(reinterpret_cast<const double2*>(a) + 1);
  return {{x.x, x.y, y.x, y.y}};
}
// the same through the coherent path, for the fields the kernel updates
__device__ __forceinline__ V4<float> ld4c(const float* a) {
  const float4 x = *reinterpret_cast<const float4*>(a);
  return {{x.x, x.y, x.z, x.w}};
}
__device__ __forceinline__ V4<double> ld4c(const double* a) {
  const double2 x = reinterpret_cast<const double2*>(a)[0], y = reinterpret_cast<const double2*>(a)[1];
  return {{x.x, x.y, y.x, y.y}};
}
__device__ __forceinline__ void st4(float* a, const V4<float>& v) {
  *reinterpret_cast<float4*>(a) = make_float4(v.v[0], v.v[1], v.v[2], v.v[3]);
}
__device__ __forceinline__ void st4(double* a, const V4<double>& v) {
  reinterpret_cast<double2*>(a)[0] = make_double2(v.v[0], v.v[1]);
  reinterpret_cast<double2*>(a)[1] = make_double2(v.v[2], v.v[3]);
}

// Coefficient k of cell j (0..3) of a core thread: from the vectors of the
// Biot planes (slots s0.. of `bio`), else through coef().
template <class T, int MODE>
__device__ __forceinline__ T core_coef(const Params<T>& p, int k, long long cell, int J, const V4<T>* bio, int s0,
                                       int j) {
  if constexpr (MODE == M_BIOT) {
    const T v = bio[biot_slot(k) - s0].v[j];
    return biot_neg(k) ? -v : v;
  } else {
    return coef<T, MODE>(p, k, cell, J);
  }
}

// Two CTAs per SM in both precisions (FP64: 128 registers, no spills; 4.50
// instead of 4.20 Gcell-updates/s with one CTA of up to 252 registers).
#define FDP_CORE_BOUNDS(T) __launch_bounds__(kBX * kBZ, 2)

// Inputs of the interior stress update of four consecutive cells of a row
// (columns I0..I0+3, row L): row L of u, w and qx as three vectors each
// (columns I0-4 .. I0+7) and the column values the z stencils need.
template <class T> struct StressCoreIn {
  V4<T> ur[3], wr[3], xr[3];
  V4<T> um2, um1, up1, wm1, wp1, wp2, zm1, z0, zp1, zp2;
};

// Loads them from velocity arrays at the field offset c0 of (I0, L).
template <class T>
__device__ __forceinline__ void load_stress_core_in(StressCoreIn<T>& a, const T* U, const T* W, const T* X,
                                                    const T* Z, long long P) {
  a.ur[0] = ld4(U - 4); a.ur[1] = ld4(U); a.ur[2] = ld4(U + 4);
  a.wr[0] = ld4(W - 4); a.wr[1] = ld4(W); a.wr[2] = ld4(W + 4);
  a.xr[0] = ld4(X - 4); a.xr[1] = ld4(X); a.xr[2] = ld4(X + 4);
  a.um2 = ld4(U - 2 * P); a.um1 = ld4(U - P); a.up1 = ld4(U + P);
  a.wm1 = ld4(W - P); a.wp1 = ld4(W + P); a.wp2 = ld4(W + 2 * P);
  a.zm1 = ld4(Z - P); a.z0 = ld4(Z); a.zp1 = ld4(Z + P); a.zp2 = ld4(Z + 2 * P);
}

// The interior stress update of the four cells (strain_uw_xz.F90:81-84,
// strain_uw_zz.F90:51,58-59, strain_q_zz.F90:48,55-56, strain_uw_xx.F90:82-83,
// strain_q_xx.F90:77-78, stress_xz.F90:44-46, stress_nn.F90:53-59): the old
// stresses o* become the new ones.  Cell src_j (0..3, or -1 for none) is
// the source cell of row LIN_Z, which adds the source term of
// stress_lin_nn.F90:58-63 (srcS = (SOURS-SOURSP)/DT, srcF the fluid one).
template <class T, int MODE>
__device__ __forceinline__ void stress_core_math(const Params<T>& p, long long c0, const StressCoreIn<T>& a,
                                                 const V4<T>* bio, V4<T>& oxz, V4<T>& oxx, V4<T>& ozz,
                                                 V4<T>& opr, int src_j = -1, T srcS = T(0), T srcF = T(0)) {
  // value of row vector r at column I0 + j + d, d in -4..7
  auto at = [](const V4<T>* r, int j, int d) { return r[(j + d + 4) >> 2].v[(j + d + 4) & 3]; };
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const long long cell_ = c0 + j;
    const int J_ = (MODE == M_TABLE) ? p.JM[cell_] : 0;
    auto C = [&](int k) { return core_coef<T, MODE>(p, k, cell_, J_, bio, 0, j); };
    // strain_uw_xz.F90:81-84
    const T exz = p.AH * (a.up1.v[j] - a.um2.v[j] + at(a.wr, j, 1) - at(a.wr, j, -2))
                + p.BH * (a.ur[1].v[j] - a.um1.v[j] + a.wr[1].v[j] - at(a.wr, j, -1));
    // strain_uw_zz.F90:51,58-59 and strain_q_zz.F90:48,55-56
    T ezz = (p.CH * (a.wp1.v[j] - a.wr[1].v[j]));
    ezz = p.AH * (a.wp2.v[j] - a.wm1.v[j]) + p.BC * ezz;
    T qzz = (p.CH * (a.zp1.v[j] - a.z0.v[j]));
    qzz = p.AH * (a.zp2.v[j] - a.zm1.v[j]) + p.BC * qzz;
    // strain_uw_xx.F90:82-83 and strain_q_xx.F90:77-78
    const T exx = p.AH * (at(a.ur, j, 2) - at(a.ur, j, -1)) + p.BH * (at(a.ur, j, 1) - a.ur[1].v[j]);
    const T qxx = p.AH * (at(a.xr, j, 2) - at(a.xr, j, -1)) + p.BH * (at(a.xr, j, 1) - a.xr[1].v[j]);
    // stress_xz.F90:44-46 and stress_nn.F90:53-59
    const T TXZv = C(C_MU) * exz;
    oxz.v[j] = oxz.v[j] + p.DTE * TXZv;
    const T s1 = C(C_SXX1), s2 = C(C_SXX2), s3 = C(C_SXX3);
    const T z1 = C(C_SZZ1), z2 = C(C_SZZ2), z3 = C(C_SZZ3);
    const T q1 = C(C_P1), q2 = C(C_P2), q3 = C(C_P3);
    const T TXXv = s1 * exx + s2 * ezz + s3 * qxx + s3 * qzz;
    const T TZZv = z1 * exx + z2 * ezz + z3 * qxx + z3 * qzz;
    const T PRv = q1 * exx + q2 * ezz + q3 * qxx + q3 * qzz;
    if (j == src_j) {
      // stress_lin_nn.F90:58-63
      oxx.v[j] = oxx.v[j] + p.DTE * (TXXv - srcS);
      ozz.v[j] = ozz.v[j] + p.DTE * (TZZv - srcS);
      opr.v[j] = opr.v[j] + p.DTE * (PRv + srcF);
    } else {
      oxx.v[j] = oxx.v[j] + p.DTE * TXXv;
      ozz.v[j] = ozz.v[j] + p.DTE * TZZv;
      opr.v[j] = opr.v[j] + p.DTE * PRv;
    }
  }
}

// core block (bx, by) of a phase: 4*kBX columns by kBZ rows of its core
template <class T, int MODE>
__device__ __forceinline__ void stress_core_block(const Params<T>& p, int bx, int by) {
  const int I0 = p.cs_x0 + 4 * (int)(bx * kBX + threadIdx.x);
  const int L = p.cs_z0 + (int)(by * kBZ + threadIdx.y);
  if (I0 >= p.cs_x1 || L >= p.cs_z1 || L == p.LIN_Z) return;
  const long long P = p.pitch;
  const long long c0 = (long long)L * P + (I0 - p.PMLL);
  // row L of u, w, qx with the vectors either side (columns I0-4 .. I0+7),
  // and the column values the z stencils need
  StressCoreIn<T> a;
  load_stress_core_in(a, p.UM + c0, p.WM + c0, p.QX + c0, p.QZ + c0, P);
  V4<T> oxz = ld4c(p.TXZ + c0), oxx = ld4c(p.TXX + c0), ozz = ld4c(p.TZZ + c0), opr = ld4c(p.PRES + c0);
  V4<T> bio[5];
  if constexpr (MODE == M_BIOT) {
#pragma unroll
    for (int s = 0; s < 5; ++s) bio[s] = ld4(p.bplane[s] + c0);
  }
  stress_core_math<T, MODE>(p, c0, a, bio, oxz, oxx, ozz, opr);
  st4(p.oTXZ + c0, oxz);
  st4(p.oTXX + c0, oxx);
  st4(p.oTZZ + c0, ozz);
  st4(p.oPRES + c0, opr);
}

template <class T, int MODE>
__global__ void FDP_CORE_BOUNDS(T) k_stress_core(const __grid_constant__ Params<T> p) {
  stress_core_block<T, MODE>(p, (int)blockIdx.x, (int)blockIdx.y);
}

// Inputs of the interior velocity update of four consecutive cells of a
// row (columns I0..I0+3, row L): row L of txx, p and txz as three vectors
// each (columns I0-4 .. I0+7) and the column values the z stencils need.
template <class T> struct VelocityCoreIn {
  V4<T> xxr[3], prr[3], xzr[3];
  V4<T> prm2, prm1, prp1, xzm1, xzp1, xzp2, zzm2, zzm1, zz0, zzp1;
};

template <class T>
__device__ __forceinline__ void load_velocity_core_in(VelocityCoreIn<T>& a, const T* XX, const T* ZZ, const T* XZ,
                                                      const T* PR, long long P) {
  a.xxr[0] = ld4(XX - 4); a.xxr[1] = ld4(XX); a.xxr[2] = ld4(XX + 4);
  a.prr[0] = ld4(PR - 4); a.prr[1] = ld4(PR); a.prr[2] = ld4(PR + 4);
  a.xzr[0] = ld4(XZ - 4); a.xzr[1] = ld4(XZ); a.xzr[2] = ld4(XZ + 4);
  a.prm2 = ld4(PR - 2 * P); a.prm1 = ld4(PR - P); a.prp1 = ld4(PR + P);
  a.xzm1 = ld4(XZ - P); a.xzp1 = ld4(XZ + P); a.xzp2 = ld4(XZ + 2 * P);
  a.zzm2 = ld4(ZZ - 2 * P); a.zzm1 = ld4(ZZ - P); a.zz0 = ld4(ZZ); a.zzp1 = ld4(ZZ + P);
}

// The interior velocity update of the four cells (inh_qx_int.F90:44-52,
// inh_v_uv_int.F90:45-54, inh_qz_int.F90:45-53, inh_v_w_int.F90:47-56),
// with the old q standing in for QXP/QZP: the old o* become the new ones.
template <class T, int MODE>
__device__ __forceinline__ void velocity_core_math(const Params<T>& p, long long c0, const VelocityCoreIn<T>& a,
                                                   const V4<T>* bio, V4<T>& oqx, V4<T>& oum, V4<T>& oqz,
                                                   V4<T>& owm) {
  const T A = p.A, B = p.B;
  auto at = [](const V4<T>* r, int j, int d) { return r[(j + d + 4) >> 2].v[(j + d + 4) & 3]; };
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const long long cell_ = c0 + j;
    const int J_ = (MODE == M_TABLE) ? p.JM[cell_] : 0;
    auto C = [&](int k) { return core_coef<T, MODE>(p, k, cell_, J_, bio, 5, j); };
    const T pr0 = a.prr[1].v[j];
    {
      // inh_qx_int.F90:44-52 and inh_v_uv_int.F90:45-54
      const T E = C(C_EQX), Cu = C(C_CU);
      const T R1 = C(C_R1QX), R2 = C(C_R2QX), R1u = C(C_R1U), R3u = C(C_R3U);
      const T qx0 = oqx.v[j], u0 = oum.v[j];
      const T Xs = A * (at(a.xxr, j, 1) - at(a.xxr, j, -2) + a.xzp2.v[j] - a.xzm1.v[j])
                 + B * (a.xxr[1].v[j] - at(a.xxr, j, -1) + a.xzp1.v[j] - a.xzr[1].v[j]);
      const T Pp = A * (at(a.prr, j, 1) - at(a.prr, j, -2)) + B * (pr0 - at(a.prr, j, -1));
      oqx.v[j] = E * qx0 - R1 * Xs - R2 * Pp;
      oum.v[j] = u0 + Cu * qx0 + R1u * Xs + R3u * Pp;
    }
    {
      // inh_qz_int.F90:45-53 and inh_v_w_int.F90:47-56
      const T E = C(C_EQZ), Cw = C(C_CW);
      const T R1 = C(C_R1QZ), R2 = C(C_R2QZ), R1w = C(C_R1W), R3w = C(C_R3W);
      const T qz0 = oqz.v[j], w0 = owm.v[j];
      const T Xs = A * (a.zzp1.v[j] - a.zzm2.v[j] + at(a.xzr, j, 2) - at(a.xzr, j, -1))
                 + B * (a.zz0.v[j] - a.zzm1.v[j] + at(a.xzr, j, 1) - a.xzr[1].v[j]);
      const T Pp = A * (a.prp1.v[j] - a.prm2.v[j]) + B * (pr0 - a.prm1.v[j]);
      oqz.v[j] = E * qz0 - R1 * Xs - R2 * Pp;
      owm.v[j] = w0 + Cw * qz0 + R1w * Xs + R3w * Pp;
    }
  }
}

template <class T, int MODE>
__device__ __forceinline__ void velocity_core_block(const Params<T>& p, int bx, int by) {
  const int I0 = p.cv_x0 + 4 * (int)(bx * kBX + threadIdx.x);
  const int L = p.cv_z0 + (int)(by * kBZ + threadIdx.y);
  if (I0 >= p.cv_x1 || L >= p.cv_z1) return;
  const long long P = p.pitch;
  const long long c0 = (long long)L * P + (I0 - p.PMLL);
  VelocityCoreIn<T> a;
  load_velocity_core_in(a, p.TXX + c0, p.TZZ + c0, p.TXZ + c0, p.PRES + c0, P);
  V4<T> oqx = ld4c(p.QX + c0), oum = ld4c(p.UM + c0), oqz = ld4c(p.QZ + c0), owm = ld4c(p.WM + c0);
  V4<T> bio[5];
  if constexpr (MODE == M_BIOT) {
#pragma unroll
    for (int s = 0; s < 5; ++s) bio[s] = ld4(p.bplane[5 + s] + c0);
  }
  velocity_core_math<T, MODE>(p, c0, a, bio, oqx, oum, oqz, owm);
  st4(p.oQX + c0, oqx);
  st4(p.oUM + c0, oum);
  st4(p.oQZ + c0, oqz);
  st4(p.oWM + c0, owm);
}

template <class T, int MODE>
__global__ void FDP_CORE_BOUNDS(T) k_velocity_core(const __grid_constant__ Params<T> p) {
  velocity_core_block<T, MODE>(p, (int)blockIdx.x, (int)blockIdx.y);
}

// Frame and core of a phase in one launch.  Blocks are dispatched in index
// order, so the frame units are spread through the grid -- one after every
// `per` core blocks -- and their latency-bound cells ride along with the
// bandwidth-bound core instead of queueing before or after it.  Block b:
// k = b / (per + 1); the first block of group k < nframe is frame unit k,
// the others are core blocks k*per .. k*per + per - 1 (those past the last
// core block do nothing).
struct FusedGrid {
  const int4* units;  // frame units of the phase
  int nframe;
  int per;            // core blocks per frame unit
  int ncore;          // core blocks
  int gx;             // core blocks along x
};

__device__ __forceinline__ int fused_role(const FusedGrid& g, int b, int& idx) {
  if (g.nframe == 0) { idx = b; return 1; }
  const int k = b / (g.per + 1), r = b % (g.per + 1);
  if (k < g.nframe && r == 0) { idx = k; return 0; }
  idx = k < g.nframe ? k * g.per + r - 1 : g.nframe * g.per + (b - g.nframe * (g.per + 1));
  return idx < g.ncore ? 1 : -1;
}

template <class T, bool SI, int MODE>
__global__ void FDP_CORE_BOUNDS(T) k_stress_fused(const __grid_constant__ Params<T> p, const FusedGrid g,
                                                  int it_off) {
  int idx;
  const int role = fused_role(g, (int)blockIdx.x, idx);
  if (role == 0) {
    const int4 u = g.units[idx];
    stress_unit<T, SI, MODE>(p, u.x, u.y, u.z, it_off);
  } else if (role == 1) {
    stress_core_block<T, MODE>(p, idx % g.gx, idx / g.gx);
  }
}

template <class T, bool SI, int MODE>
__global__ void FDP_CORE_BOUNDS(T) k_velocity_fused(const __grid_constant__ Params<T> p, const FusedGrid g) {
  int idx;
  const int role = fused_role(g, (int)blockIdx.x, idx);
  if (role == 0) velocity_frame_unit<T, SI, MODE>(p, g.units[idx]);
  else if (role == 1) velocity_core_block<T, MODE>(p, idx % g.gx, idx / g.gx);
}

// ---------------------------------------------------------------------------
// Stress-imaging row 1 (inh_v_qx_int_1_si.F90:26-31, inh_w_qz_int_1_si.F90:30-44),
// from the final rows 2 and 3.  Returns the row-1 value of u (c=0), w (1),
// qx (2) or qz (3) at column I, or the stored value where row 1 is not updated.
template <class T>
__device__ __forceinline__ T si_row1(const Params<T>& p, int c, int I) {
  const int TPML = p.TPML, MX = p.MX;
  auto u1 = [&](int i) { return FDP_F(p.UM, i, 2) + FDP_F(p.WM, i, 2) - FDP_F(p.WM, i - 1, 2); };
  auto q1 = [&](int i) { return FDP_F(p.QX, i, 2) + FDP_F(p.QZ, i, 2) - FDP_F(p.QZ, i - 1, 2); };
  if (c == 0) return (I >= 3 - TPML && I <= MX - 1 + TPML) ? u1(I) : FDP_F(p.UM, I, 1);
  if (c == 2) return (I >= 3 - TPML && I <= MX - 1 + TPML) ? q1(I) : FDP_F(p.QX, I, 1);
  if (I < 3 - TPML || I > MX - 2 + TPML) return c == 1 ? FDP_F(p.WM, I, 1) : FDP_F(p.QZ, I, 1);
  const T du = u1(I + 1) - u1(I) + FDP_F(p.UM, I + 1, 2) - FDP_F(p.UM, I, 2);
  const int x = I - p.PMLL;  // AUX holds AUXIL_W/AUXIL_QZ of material JM(I,0)
  if (c == 1) return FDP_F(p.WM, I, 3) + p.AUX[x] * du;
  return FDP_F(p.QZ, I, 3) + p.AUX[p.NX + x] * du + (q1(I + 1) - q1(I) + FDP_F(p.QX, I + 1, 2) - FDP_F(p.QX, I, 2));
}

template <class T, bool SI>
__device__ __forceinline__ T final_value(const Params<T>& p, int c, int I, int L) {
  if (SI && L == 1) return si_row1(p, c, I);
  const T* f = c == 0 ? p.UM : c == 1 ? p.WM : c == 2 ? p.QX : p.QZ;
  return FDP_F(f, I, L);
}

// Row 1 under stress imaging (threads 0..NX-1) and receiver sampling (the
// next MR threads): no thread does both, so neither chain of loads waits
// for the other.
// Sampling recomputes row-1 values instead of reading them, so it does not
// depend on the order in which threads write row 1.
// g is the thread's index within the shot.
template <class T, bool SI>
__device__ __forceinline__ void edge_thread(const Params<T>& p, int g, int it_off) {
  const int nsi = SI ? p.NX : 0;  // threads 0..nsi-1: row 1; the next MR: receivers
  if (g < nsi) {
    const int I = p.PMLL + g;
    if (I <= p.PMLXH && I >= 3 - p.TPML && I <= p.MX - 1 + p.TPML) {
      const T u = si_row1(p, 0, I), qx = si_row1(p, 2, I);
      T w = T(0), qz = T(0);
      const bool wq = (I <= p.MX - 2 + p.TPML);
      if (wq) { w = si_row1(p, 1, I); qz = si_row1(p, 3, I); }
      // all reads of row 1 above come before any write; another thread's
      // row-1 cells are recomputed from rows 2 and 3, never read
      FDP_F(p.UM, I, 1) = u;
      FDP_F(p.QX, I, 1) = qx;
      if (wq) { FDP_F(p.WM, I, 1) = w; FDP_F(p.QZ, I, 1) = qz; }
    }
  }
  g -= nsi;
  if (g >= 0 && g < p.MR) {
    const int it = *p.it_base + it_off;
    const int IX = p.REC[4 * g], LX = p.REC[4 * g + 1], IZ = p.REC[4 * g + 2], LZ = p.REC[4 * g + 3];
    auto inside = [&](int i, int l) { return i >= p.PMLL && i <= p.PMLXH && l >= 0 && l <= p.PMLZH; };
    T s[4] = {T(0), T(0), T(0), T(0)};
    if (inside(IX, LX)) { s[0] = final_value<T, SI>(p, 0, IX, LX); s[2] = final_value<T, SI>(p, 2, IX, LX); }
    if (inside(IZ, LZ)) { s[1] = -final_value<T, SI>(p, 1, IZ, LZ); s[3] = -final_value<T, SI>(p, 3, IZ, LZ); }
    T* out = p.RAW + ((long long)(it - 1) * p.MR + g) * 6;
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = s[k];
  }
}

// The stress samples of receiver g (store_seismograms_pressure.F90:45-58):
// p and -txx at (IRECZ, LRECX).  The velocity phase leaves the stresses
// alone, so they can be taken any time after the stress phase.
template <class T>
__device__ __forceinline__ void stress_sample_thread(const Params<T>& p, int g, int it_off) {
  if (g < 0 || g >= p.MR) return;
  const int it = *p.it_base + it_off;
  const int LX = p.REC[4 * g + 1], IZ = p.REC[4 * g + 2];
  const bool in = IZ >= p.PMLL && IZ <= p.PMLXH && LX >= 0 && LX <= p.PMLZH;
  T* out = p.RAW + ((long long)(it - 1) * p.MR + g) * 6;
  out[4] = in ? FDP_F(p.PRES, IZ, LX) : T(0);
  out[5] = in ? -FDP_F(p.TXX, IZ, LX) : T(0);
}

// samples = 0 leaves the stress samples to the velocity frame kernel.
template <class T, bool SI>
__global__ void __launch_bounds__(128) k_edge(const __grid_constant__ Params<T> p, int it_off, int samples) {
  const int g = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  edge_thread<T, SI>(p, g, it_off);
  if (samples) stress_sample_thread<T>(p, g - (SI ? p.NX : 0), it_off);
}

// ---------------------------------------------------------------------------
// Batched shots.  Every shot of a batch advances one level per launch of
// each kernel.  A kernel's work is a queue of items, taken round-robin by
// persistent CTAs that hold the current shot's parameters in shared memory:
// without a core (framed = 0), an item of a cell phase is `m` vertically
// adjacent units of one shot's grid; with the frame/core split, a frame
// item is one listed frame unit of a shot and a core item `m` vertically
// adjacent core blocks; an edge item is kBX * kBZ consecutive edge threads.
// Shots may differ in grid size, medium, source and receivers, and share
// precision, free-surface mode and medium representation.
struct BatchQueue {
  const void* params;  // Params<T>[n]
  const int* first;    // [5][n+1]: first item of each shot: stress, velocity, edge, stress core, velocity core
  const int4* units;   // frame units (first column, end column, unit row) of every shot and phase
  const int* ubase;    // [2][n]: offset in `units` of shot s's stress / velocity frame units
  int n;               // shots
  int m;               // units (core blocks) per cell item
  int framed;          // 1: frame/core split
};

// largest s with first[s] <= item (first[0] = 0, first[n] = items)
__device__ __forceinline__ int batch_shot(const int* first, int n, int item) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(first + mid) <= item) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <class T>
__device__ __forceinline__ void batch_load_params(Params<T>& dst, const BatchQueue& q, int s) {
  static_assert(sizeof(Params<T>) % 4 == 0, "parameter block is copied as 32-bit words");
  const int* src = (const int*)((const Params<T>*)q.params + s);
  int* d = (int*)&dst;
  const int tid = (int)(threadIdx.y * blockDim.x + threadIdx.x);
  for (int k = tid; k < (int)(sizeof(Params<T>) / 4); k += (int)(blockDim.x * blockDim.y)) d[k] = __ldg(src + k);
}

// units (phase 0 stress, 1 velocity) or core blocks (2 stress, 3 velocity)
// along x and y of a shot's grid
template <class T>
__device__ __forceinline__ int2 batch_units(const Params<T>& p, int phase) {
  if (phase >= 2) {
    const int x0 = phase == 2 ? p.cs_x0 : p.cv_x0, x1 = phase == 2 ? p.cs_x1 : p.cv_x1;
    const int z0 = phase == 2 ? p.cs_z0 : p.cv_z0, z1 = phase == 2 ? p.cs_z1 : p.cv_z1;
    return make_int2(((x1 - x0) / 4 + kBX - 1) / kBX, (z1 - z0 + kBZ - 1) / kBZ);
  }
  const int rows = kBZ * (phase == 0 ? kRZS : kRZV);
  return make_int2((p.NX + kBX - 1) / kBX, (p.PMLZH + 1 + rows - 1) / rows);
}

// PHASE 0/1: units (all of them, or the listed frame units); 2/3: core blocks
template <class T, bool SI, int MODE, int PHASE>
__device__ __forceinline__ void batch_cells(const BatchQueue& q, int items, int it_off) {
  __shared__ Params<T> sp;
  // queues: 0 stress, 1 velocity, 2 edge, 3 stress core, 4 velocity core
  const int* first = q.first + (PHASE < 2 ? PHASE : PHASE + 1) * (q.n + 1);
  int cur = -1;
  for (int item = (int)blockIdx.x; item < items; item += (int)gridDim.x) {
    const int s = batch_shot(first, q.n, item);
    if (s != cur) {
      __syncthreads();  // the previous shot's parameters are no longer read
      batch_load_params<T>(sp, q, s);
      __syncthreads();
      cur = s;
    }
    const int j = item - __ldg(first + s);
    if (PHASE < 2 && q.framed) {
      const int4 u = q.units[__ldg(q.ubase + PHASE * q.n + s) + j];
      if (PHASE == 0) stress_unit<T, SI, MODE>(sp, u.x, u.y, u.z, it_off);
      else velocity_frame_unit<T, SI, MODE>(sp, u);
      continue;
    }
    const int2 g = batch_units(sp, PHASE);
    const int bx = j % g.x, by0 = (j / g.x) * q.m;
    const int by1 = min(by0 + q.m, g.y);
    for (int by = by0; by < by1; ++by) {
      if (PHASE == 0) stress_unit<T, SI, MODE>(sp, sp.PMLL + bx * kBX, sp.PMLXH + 1, by, it_off);
      else if (PHASE == 1) velocity_unit<T, SI, MODE>(sp, sp.PMLL + bx * kBX, sp.PMLXH + 1, by);
      else if (PHASE == 2) stress_core_block<T, MODE>(sp, bx, by);
      else velocity_core_block<T, MODE>(sp, bx, by);
    }
  }
}

template <class T, bool SI, int MODE>
__global__ void __launch_bounds__(kBX * kBZ) k_stress_batch(const __grid_constant__ BatchQueue q, int items, int it_off) {
  batch_cells<T, SI, MODE, 0>(q, items, it_off);
}

template <class T, bool SI, int MODE>
__global__ void FDP_VELOCITY_BOUNDS(T) k_velocity_batch(const __grid_constant__ BatchQueue q, int items, int it_off) {
  batch_cells<T, SI, MODE, 1>(q, items, it_off);
}

template <class T, int MODE>
__global__ void FDP_CORE_BOUNDS(T) k_stress_core_batch(const __grid_constant__ BatchQueue q, int items) {
  batch_cells<T, false, MODE, 2>(q, items, 0);
}

template <class T, int MODE>
__global__ void FDP_CORE_BOUNDS(T) k_velocity_core_batch(const __grid_constant__ BatchQueue q, int items) {
  batch_cells<T, false, MODE, 3>(q, items, 0);
}

template <class T, bool SI>
__global__ void __launch_bounds__(kBX * kBZ) k_edge_batch(const __grid_constant__ BatchQueue q, int items, int it_off) {
  __shared__ Params<T> sp;
  const int* first = q.first + 2 * (q.n + 1);
  const int tid = (int)(threadIdx.y * blockDim.x + threadIdx.x);
  int cur = -1;
  for (int item = (int)blockIdx.x; item < items; item += (int)gridDim.x) {
    const int s = batch_shot(first, q.n, item);
    if (s != cur) {
      __syncthreads();
      batch_load_params<T>(sp, q, s);
      __syncthreads();
      cur = s;
    }
    const int g = (item - __ldg(first + s)) * (kBX * kBZ) + tid;
    edge_thread<T, SI>(sp, g, it_off);
    stress_sample_thread<T>(sp, g - (SI ? sp.NX : 0), it_off);
  }
}

// ---------------------------------------------------------------------------
// TMA-staged variants of the two phases.
//
// A CTA of 64 x 4 threads owns a tile of kTX x kTZ cells.  One thread issues
// a 2-D bulk tensor copy (cp.async.bulk.tensor) of each of the phase's four
// input fields -- the tile plus kHX columns and kHZ rows of halo -- into
// shared memory, completing on one mbarrier; meanwhile every thread
// prefetches the cells it read-modify-writes and their medium planes into
// L1.  Each thread then updates kRows cells of one column with every stencil
// neighbour read from shared memory.  The cell arithmetic is the same
// stress_cell / velocity_cell code as the global-load kernels.
constexpr int kTX = 64, kTZ = 16, kHX = 4, kHZ = 2;
constexpr int kSX = kTX + 2 * kHX, kSZ = kTZ + 2 * kHZ;
constexpr int kRows = kTZ / 4;
static_assert(kHX == kPadX, "the halo of a tile must start on the 16-byte-aligned padding column");

struct TmaMaps {
  CUtensorMap m[4];  // the phase's input fields, boxes of kSX x kSZ elements
};

template <class T> struct SmemRd {
  const T* s;  // [4][kSZ][kSX]
  int I0, L0;  // cell of tile element (kHX, kHZ)
  __device__ __forceinline__ T operator()(int k, int I, int L) const {
    return s[(k * kSZ + (L - L0 + kHZ)) * kSX + (I - I0 + kHX)];
  }
};

__device__ __forceinline__ uint32_t smem_u32(const void* ptr) { return (uint32_t)__cvta_generic_to_shared(ptr); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// The failure path of the bounded waits, on its own: polls a word that
// nothing sets, `polls` times about 100 ns apart, then records the expired
// wait in the status word the host reads, as a kernel whose tile copy does
// not arrive does.
static __global__ void k_wait_flag(const int* flag, unsigned polls, int* err) {
  for (unsigned i = 0; i < polls; ++i) {
    if (*(const volatile int*)flag) return;
    __nanosleep(100);
  }
  atomicOr(err, 4);
}

// Waits for the tile's copies with an iteration limit (far above any real
// latency); false means the copies did not complete in time.
constexpr unsigned kWaitLimit = 1u << 22;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (unsigned i = 0; i < kWaitLimit; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_u32(dst)),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void prefetch_l1(const void* ptr) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(ptr));
}

// Issues the tile copy (thread 0), prefetches the thread's own cells, and
// waits.  x, y: element coordinates of the tile's first halo element.
template <class T>
__device__ __forceinline__ bool stage_tile(T* s, uint64_t* bar, const TmaMaps& maps, int x, int y) {
  const int tid = threadIdx.y * kTX + threadIdx.x;
  if (tid == 0) mbar_init(bar, 1);
  __syncthreads();
  if (tid == 0) {
    mbar_expect_tx(bar, 4u * kSZ * kSX * (uint32_t)sizeof(T));
#pragma unroll
    for (int f = 0; f < 4; ++f) tma_load_2d(s + f * kSZ * kSX, &maps.m[f], x, y, bar);
  }
  return true;
}

template <class T, bool SI, int MODE>
__global__ void __launch_bounds__(kTX * 4) k_stress_tma(const __grid_constant__ Params<T> p,
                                                        const __grid_constant__ TmaMaps maps, int it_off) {
  __shared__ alignas(128) T s[4 * kSZ * kSX];
  __shared__ alignas(8) uint64_t bar;
  const int I0 = p.PMLL + (int)blockIdx.x * kTX, L0 = (int)blockIdx.y * kTZ;
  const int I = I0 + (int)threadIdx.x;
  const int Lt = L0 + (int)threadIdx.y * kRows;
  stage_tile(s, &bar, maps, (int)blockIdx.x * kTX + kPadX - kHX, L0 + kPadZ - kHZ);
  if (I <= p.PMLXH) {
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
      if (Lt + r > p.PMLZH) break;
      const long long c = (long long)(Lt + r) * p.pitch + (I - p.PMLL);
      prefetch_l1(p.TXX + c); prefetch_l1(p.TZZ + c); prefetch_l1(p.TXZ + c); prefetch_l1(p.PRES + c);
      if (MODE == M_PLANES)
        for (int k = 0; k < C_NCOEF; ++k)
          if (k <= C_P3 && p.src[k] >= 0) prefetch_l1(p.planes + (long long)p.src[k] * p.pstride + c);
    }
  }
  const int it = *p.it_base + it_off;
  const bool ok = mbar_wait_bounded(&bar, 0);
  if (!ok && threadIdx.x == 0 && threadIdx.y == 0) atomicOr(p.err, 1);
  if (ok && I <= p.PMLXH) {
    const SmemRd<T> rd{s, I0, L0};
    for (int r = 0; r < kRows; ++r) {
      const int L = Lt + r;
      if (L <= p.PMLZH && (!SI || L >= 2)) stress_cell<T, SI, MODE>(p, rd, I, L, it);
    }
  }
  if (SI && blockIdx.y == 0) {
    __syncthreads();  // rows 2..4 of this tile are final
    if (ok && I <= p.PMLXH && threadIdx.y == 0) {
      // hplane_0_stress.F90:49-53 and hplane_1_stress.F90:45-53
      stress_mirror(p, I);
    }
  }
  if (!ok) mbar_wait_bounded(&bar, 0);  // let copies still in flight land before the CTA exits
}

// Tiles run from the bottom row up, so the thread that owns the bottom row
// of a column also owns rows PMLZH-1 and PMLZH-2 (kRows >= 3) and keeps their
// pre-phase values (the history of time_loop.F90:133-155) in registers.
template <class T, bool SI, int MODE>
__global__ void __launch_bounds__(kTX * 4) k_velocity_tma(const __grid_constant__ Params<T> p,
                                                          const __grid_constant__ TmaMaps maps, int it_off) {
  static_assert(kRows >= 3, "the bottom row needs two rows above it in the same thread");
  (void)it_off;
  __shared__ alignas(128) T s[4 * kSZ * kSX];
  __shared__ alignas(8) uint64_t bar;
  const int I0 = p.PMLL + (int)blockIdx.x * kTX;
  const int L0 = p.PMLZH + 1 - ((int)blockIdx.y + 1) * kTZ;
  const int I = I0 + (int)threadIdx.x;
  const int Lt = L0 + (int)threadIdx.y * kRows;
  const int Lmin = SI ? 2 : 0;
  stage_tile(s, &bar, maps, (int)blockIdx.x * kTX + kPadX - kHX, L0 + kPadZ - kHZ);
  if (I <= p.PMLXH) {
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
      if (Lt + r < Lmin) continue;
      const long long c = (long long)(Lt + r) * p.pitch + (I - p.PMLL);
      prefetch_l1(p.UM + c); prefetch_l1(p.WM + c); prefetch_l1(p.QX + c); prefetch_l1(p.QZ + c);
      if (MODE == M_PLANES)
        for (int k = C_EQX; k <= C_R3W; ++k)
          if (p.src[k] >= 0) prefetch_l1(p.planes + (long long)p.src[k] * p.pstride + c);
    }
  }
  const bool ok = mbar_wait_bounded(&bar, 0);
  if (!ok && threadIdx.x == 0 && threadIdx.y == 0) atomicOr(p.err, 1);
  if (ok && I <= p.PMLXH) {
    const SmemRd<T> rd{s, I0, L0};
    const bool owns_bottom = (Lt + kRows - 1 == p.PMLZH);
    T old[3][4];  // pre-phase rows PMLZH (k=0), PMLZH-1 (1), PMLZH-2 (2) of u w qx qz
#pragma unroll
    for (int r = 0; r < kRows; ++r) {
      const int L = Lt + r;
      if (owns_bottom && r >= kRows - 3) {
        const int k = kRows - 1 - r;
        old[k][0] = FDP_F(p.UM, I, L); old[k][1] = FDP_F(p.WM, I, L);
        old[k][2] = FDP_F(p.QX, I, L); old[k][3] = FDP_F(p.QZ, I, L);
      }
      if (L >= Lmin && L < p.PMLZH) {
        if (!SI && L <= 1) {
          // rows 0 and 1 without stress imaging reach rows up to 4
          // (inh_qx_int_0.F90), beyond the tile's halo when the tile starts
          // above row -13
          const GlobalRd<T> grd{{p.TXX, p.TZZ, p.TXZ, p.PRES}, p.pitch, p.PMLL};
          velocity_cell<T, SI, MODE>(p, grd, I, L);
        } else {
          velocity_cell<T, SI, MODE>(p, rd, I, L);
        }
      }
    }
    if (owns_bottom) {
      // hplane_pmlzh0_velocity.F90:34-63
      const int LST = p.PMLZH, x = I - p.PMLL;
      T* const f[4] = {p.oUM, p.oWM, p.oQX, p.oQZ};  // this phase's new values
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const T* ab = p.AB + ((c == 0 || c == 2) ? 8 : 0);  // ABH for u, qx; ABW for w, qz
        T* hist = p.HIST + (long long)c * 3 * p.NX;
        const T sp0 = hist[x], sp1 = hist[p.NX + x], sp2 = hist[2 * p.NX + x];
        const T v = ab[0] * FDP_F(f[c], I, LST - 1) + ab[1] * FDP_F(f[c], I, LST - 2)
                  + ab[2] * old[0][c] + ab[3] * old[1][c] + ab[4] * old[2][c]
                  + ab[5] * sp0 + ab[6] * sp1 + ab[7] * sp2;
        FDP_F(f[c], I, LST) = v;
        hist[x] = old[0][c];
        hist[p.NX + x] = old[1][c];
        hist[2 * p.NX + x] = old[2][c];
      }
    }
  }
  if (!ok) mbar_wait_bounded(&bar, 0);
}

static __global__ void k_set_base(int* base, int v) { *base = v; }
static __global__ void k_add_base(int* base, int v) { *base += v; }

#undef FDP_F
#undef FDP_R
#undef FDP_C

}  // namespace fdp
