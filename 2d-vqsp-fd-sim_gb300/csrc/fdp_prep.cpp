// Host-side set-up of the time-stepping inputs (declared in include/fdp_prep.h).
//
// Restates, in the reference's working precision PP and evaluation order,
// the set-up routines the Fortran driver runs before TIME_LOOP.  Literals
// that are default-real in the reference stay single precision here too
// (e.g. 0.075 in ppml.F90:183 becomes (T)0.075f), which is what a PP=DP
// build of the reference computes.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "fdp.h"
#include "fdp_prep.h"

namespace {

// .MO record column order (read_model_par.F90:52-60)
enum { MU, SXX1, SXX2, SXX3, SZZ1, SZZ2, SZZ3, P1, P2, P3, R1U, R1W, R2U, R2W, R3U, R3W,
       R1QX, R1QZ, R2QX, R2QZ, R3QX, R3QZ, AUXW, AUXQZ };

// calcul_velocity.F90:16-36
template <class T>
void calcul_velocity(T SIG_1, T P, T AINV, T MU_, T REL1, T REL2, T REL3, T& VPF, T& VPS, T& VS) {
  const T A11 = REL1, A22 = REL2, A12 = -REL3, A21 = -REL3;
  const T B11 = SIG_1, B22 = AINV, B12 = P, B21 = P;
  // TT = MATMUL(AINVER, B)
  const T T11 = A11 * B11 + A12 * B21;
  const T T12 = A11 * B12 + A12 * B22;
  const T T21 = A21 * B11 + A22 * B21;
  const T T22 = A21 * B12 + A22 * B22;
  const T DELTA = (T11 + T22) * (T11 + T22) + T(4) * (T12 * T21 - T11 * T22);
  const T D1 = ((T11 + T22) + std::sqrt(DELTA)) / T(2);
  const T D2 = ((T11 + T22) - std::sqrt(DELTA)) / T(2);
  VPF = std::sqrt(D1);
  VPS = std::sqrt(D2);
  VS = std::sqrt(REL1 * MU_);
  if (MU_ == T(0)) VS = VPF;
}

// Velocities used by PPML's x-profiles and PRE_NR_COEF1 (ppml.F90:168,215;
// pre_nr_coef1.F90:190): solid coefficients of the x-direction.
template <class T> void vel_x(const T* r, T H, T DT, T& vpf, T& vps, T& vs) {
  calcul_velocity<T>(r[SXX1], -r[P1], -r[P3], r[MU], H * r[R1U] / DT, H * r[R2QX] / DT, H * r[R3U] / DT, vpf, vps, vs);
}
// ... and of the z-direction (ppml.F90:265, open_sr_file.F90:46)
template <class T> void vel_z(const T* r, T H, T DT, T& vpf, T& vps, T& vs) {
  calcul_velocity<T>(r[SZZ2], -r[P2], -r[P3], r[MU], H * r[R1W] / DT, H * r[R2QZ] / DT, H * r[R3W] / DT, vpf, vps, vs);
}

// One profile column of ppml.F90:171-207: J = 0..TPML for OD*, 0..TPML+1 for OD2*.
template <class T>
void profile(T OMG, T VEL, T POW, T SF, T WC, T DT, int TPML, T* oda, T* odb, T* odc, T* odd, T* oda2, T* odb2,
             T* odc2, T* odd2) {
  for (int J = 0; J <= TPML; ++J) { oda[J] = T(1); odb[J] = T(1); odc[J] = T(0); }
  for (int J = 0; J <= TPML + 1; ++J) { oda2[J] = T(1); odb2[J] = T(1); odc2[J] = T(0); }
  auto one = [&](T OMGPDT, T& a, T& b, T& c) {
    const T AP = T(1) + SF * OMGPDT * (T)0.075f / (T)0.91f;
    const T DENOM = std::exp(-OMGPDT / AP - WC * DT);
    a = (DENOM + T(1)) / T(2) / AP;
    b = DENOM;
    c = OMGPDT / (OMGPDT + WC * AP * DT) * (DENOM - T(1));
  };
  for (int J = 1; J <= TPML; ++J) {
    one(OMG * VEL * std::pow((T)(float)J, POW), oda[J], odb[J], odc[J]);
    one(OMG * VEL * std::pow((T)((float)J - 0.5f), POW), oda2[J], odb2[J], odc2[J]);
  }
  const int J = TPML + 1;
  one(OMG * VEL * std::pow((T)((float)J - 0.5f), POW), oda2[J], odb2[J], odc2[J]);
  for (int K = 0; K <= TPML; ++K) odd[K] = (odc[K] + T(2)) / (odb[K] + T(1));
  for (int K = 0; K <= TPML + 1; ++K) odd2[K] = (odc2[K] + T(2)) / (odb2[K] + T(1));
}

template <class T>
int pml_t(int MX, int MZ, int TPML, int KTBO, T R, T TAU, T POW, T SF, T WC, T DT, T H, const int32_t* jm,
          int jmnum, const T* tab, void* const* out) {
  const int PMLL = 1 - TPML, PMLXH = MX + TPML, PMLZH = MZ + TPML;
  const int NX = PMLXH - PMLL + 1, NZ = PMLZH + 1;
  T* o[24];
  for (int k = 0; k < 24; ++k) o[k] = (T*)out[k];
  auto JM = [&](int I, int L) { return jm[(size_t)(I - PMLL) + (size_t)L * NX]; };
  // ppml.F90:156-160
  T OMG = (TPML == 0) ? T(0) : -TAU * std::log(R) * DT / (T)(float)TPML / std::pow((T)(float)TPML, POW) / H;
  std::vector<T> oda(TPML + 2), odb(TPML + 2), odc(TPML + 2), odd(TPML + 2);
  std::vector<T> oda2(TPML + 2), odb2(TPML + 2), odc2(TPML + 2), odd2(TPML + 2);
  for (int L = 0; L <= PMLZH; ++L) {
    for (int side = 0; side < 2; ++side) {
      const int J1 = JM(side == 0 ? PMLL : PMLXH, L);
      if (J1 < 1 || J1 > jmnum) return FDP_ERR_ARG;
      T vpf, vps, vs;
      vel_x<T>(tab + (size_t)(J1 - 1) * 24, H, DT, vpf, vps, vs);
      profile<T>(OMG, vs, POW, SF, WC, DT, TPML, oda.data(), odb.data(), odc.data(), odd.data(), oda2.data(),
                 odb2.data(), odc2.data(), odd2.data());
      const int b1 = side == 0 ? 0 : 4, b2 = side == 0 ? 12 : 16;
      for (int J = 0; J <= TPML; ++J) {
        const size_t ix = (size_t)J + (size_t)L * (TPML + 1);
        o[b1 + 0][ix] = oda[J]; o[b1 + 1][ix] = odb[J]; o[b1 + 2][ix] = odc[J]; o[b1 + 3][ix] = odd[J];
      }
      for (int J = 0; J <= TPML + 1; ++J) {
        const size_t ix = (size_t)J + (size_t)L * (TPML + 2);
        o[b2 + 0][ix] = oda2[J]; o[b2 + 1][ix] = odb2[J]; o[b2 + 2][ix] = odc2[J]; o[b2 + 3][ix] = odd2[J];
      }
    }
  }
  // ppml.F90:261-306
  if (KTBO != 0) OMG = T(0);
  for (int I = PMLL; I <= PMLXH; ++I) {
    const int J1 = JM(I, PMLZH);
    if (J1 < 1 || J1 > jmnum) return FDP_ERR_ARG;
    T vpf, vps, vs;
    vel_z<T>(tab + (size_t)(J1 - 1) * 24, H, DT, vpf, vps, vs);
    profile<T>(OMG, vpf, POW, SF, WC, DT, TPML, oda.data(), odb.data(), odc.data(), odd.data(), oda2.data(),
               odb2.data(), odc2.data(), odd2.data());
    for (int J = 0; J <= TPML; ++J) {
      const size_t ix = (size_t)J + (size_t)(I - PMLL) * (TPML + 1);
      o[8][ix] = oda[J]; o[9][ix] = odb[J]; o[10][ix] = odc[J]; o[11][ix] = odd[J];
    }
    for (int J = 0; J <= TPML + 1; ++J) {
      const size_t ix = (size_t)J + (size_t)(I - PMLL) * (TPML + 2);
      o[20][ix] = oda2[J]; o[21][ix] = odb2[J]; o[22][ix] = odc2[J]; o[23][ix] = odd2[J];
    }
  }
  (void)NZ;
  return FDP_OK;
}

// higdon_fd.F90:17-44
template <class T> void higdon_fd(T WB, T ALFA, T BETA, T DT, T H, double a[9]) {
  const double wb = (double)WB;
  const double BE1 = 1.0;
  const double BE2 = (double)ALFA / (double)BETA;
  const double NI = (double)ALFA * (double)DT / (double)H;
  const double QX = (wb * (BE1 + NI) - NI) / (BE1 + NI) / (1.0 - wb);
  const double RX = (wb * (BE2 + NI) - NI) / (BE2 + NI) / (1.0 - wb);
  const double QT = (wb * (BE1 + NI) - BE1) / (BE1 + NI) / (1.0 - wb);
  const double RT = (wb * (BE2 + NI) - BE1) / (BE2 + NI) / (1.0 - wb);
  const double QXT = wb / (wb - 1.0), RXT = wb / (wb - 1.0);
  a[0] = 0.0;
  a[1] = -(QX + RX);
  a[3] = -(QT + RT);
  a[2] = -QX * RX;
  a[6] = -QT * RT;
  a[4] = -(QX * RT + QT * RX + QXT + RXT);
  a[5] = -(QX * RXT + RX * QXT);
  a[7] = -(QT * RXT + RT * QXT);
  a[8] = -QXT * RXT;
}

// higdce_fd.F90:16-40 (GP, GS and 1-WB evaluated in PP as written)
template <class T> void higce_fd(T WB, T ALFA, T BETA, T DT, T H, double a[9]) {
  const double GP = (double)(ALFA * DT / H);
  const double GS = (double)(BETA * DT / H);
  const double GS1 = 1.0 + GS;
  const double omw = (double)(T(1) - WB);
  const double wb = (double)WB;
  const double H1X = (GS - wb * GS1) / (GS1 * omw);
  const double H1T = (1.0 - wb * GS1) / (GS1 * omw);
  const double HXT = wb / (1.0 - wb);
  const double C1T = 1.0 - GP, CXT = GP;
  a[0] = 0.0;
  a[1] = H1X;
  a[2] = 0.0;
  a[3] = C1T + H1T;
  a[4] = CXT + HXT - H1X * C1T;
  a[5] = -H1X * CXT;
  a[6] = -H1T * C1T;
  a[7] = -HXT * C1T - H1T * CXT;
  a[8] = -HXT * CXT;
}

// higdce2_fd.F90:18-43
template <class T> void higce2_fd(T WB, T VELH, T VELCE, T DT, T H, double a[9]) {
  const double wb = (double)WB;
  const double NI = (double)VELH * (double)DT / (double)H;
  const double G = (double)VELCE * (double)DT / (double)H;
  const double QX = (wb * (1.0 + NI) - NI) / (1.0 + NI) / (1.0 - wb);
  const double RX = (1.0 - G) / (1.0 + G);
  const double QT = (wb * (1.0 + NI) - 1.0) / (1.0 + NI) / (1.0 - wb);
  const double RT = -(1.0 - G) / (1.0 + G);
  const double QXT = wb / (wb - 1.0), RXT = -1.0;
  a[0] = 0.0;
  a[1] = -(QX + RX);
  a[3] = -(QT + RT);
  a[2] = -QX * RX;
  a[6] = -QT * RT;
  a[4] = -(QX * RT + QT * RX + QXT + RXT);
  a[5] = -(QX * RXT + RX * QXT);
  a[7] = -(QT * RXT + RT * QXT);
  a[8] = -QXT * RXT;
}

// OptAbsBc.F90:37-104 (Peng & Toksoz optimal absorbing condition, double precision)
void opt_abs_bc(double gplus, double gminus, double dt, double dx, double a[9]) {
  const double tplus = dx * std::cos(gplus), tminus = dx * std::cos(gminus);
  const double Rz = std::cos(dt), Iz = std::sin(dt);
  const double Rx = std::cos(tplus + tminus), Ix = std::sin(tplus + tminus);
  const double Ry = -(std::cos(tplus) + std::cos(tminus));
  const double Iy = -(std::sin(tplus) + std::sin(tminus));
  double temp1 = Rx * Rz - Ix * Iz;
  double temp2 = Rx * Iz + Rz * Ix;
  const double temp3 = Ry * Rz - Iy * Iz;
  const double temp4 = Ry * Iz + Rz * Iy;
  double delta = (Ry + Iy + 2.0 * Rz) * (temp1 + temp2 - Rz + Iz) + (1.0 - Rx - Ix) * (2.0 + temp3 + temp4);
  delta = 1.0 / delta;
  double r0[3][3], r1[3][3];
  r1[1][0] = (1.0 - Rz) * (temp1 + temp2 - Rz + Iz) * delta;
  r1[0][2] = (1.0 - Rz) * (1.0 - Rx - Ix) * delta;
  r1[0][1] = -0.50 - r1[1][0];
  r1[1][1] = 1.0 - 2.0 * r1[0][2];
  r1[0][0] = 0.0;
  r1[2][2] = 0.0;
  r1[1][2] = r1[1][0];
  r1[2][0] = r1[0][2];
  r1[2][1] = r1[0][1];
  const double temp5 = Rx * Rz + Ix * Iz;
  const double temp6 = Rx * Iz - Rz * Ix;
  const double temp7 = Ry * Rz + Iy * Iz;
  const double temp8 = Ry * Iz - Rz * Iy;
  const double phi = -(Rz + Iz - temp5 + temp6) * (Ry + Iy + 2.0 * Rz) + (1.0 + Rz + temp7 - temp8) * (1.0 - Rx - Ix);
  r0[0][2] = phi * delta;
  const double psi = (1.0 + Rz + temp7 - temp8) * (temp1 + temp2 - Rz + Iz) + (Rz + Iz - temp5 + temp6) * (2.0 + temp3 + temp4);
  r0[1][0] = psi * delta;
  r0[0][0] = 0.0;
  r0[0][1] = 0.50 - r0[1][0];
  r0[1][1] = 1.0 - 2.0 * r0[0][2];
  r0[2][2] = -1.0;
  r0[1][2] = r0[1][0];
  r0[2][0] = r0[0][2];
  r0[2][1] = r0[0][1];
  temp1 = 0.0;
  temp2 = 0.0;
  // Fortran r0(i,j) loop order: i outer, j inner
  for (int i = 0; i <= 2; ++i)
    for (int j = 0; j <= 2; ++j) {
      temp1 = temp1 + r0[i][j] * r1[i][j];
      temp2 = temp2 + r1[i][j] * r1[i][j];
    }
  const double ratio = -temp1 / temp2;
  a[0] = 0.0;
  a[1] = r0[0][1] + ratio * r1[0][1];
  a[2] = r0[0][2] + ratio * r1[0][2];
  a[3] = r0[1][0] + ratio * r1[1][0];
  a[4] = r0[1][1] + ratio * r1[1][1];
  a[5] = r0[1][2] + ratio * r1[1][2];
  a[6] = r0[2][0] + ratio * r1[2][0];
  a[7] = r0[2][1] + ratio * r1[2][1];
  a[8] = r0[2][2] + ratio * r1[2][2];
}

// nonref.F90:69-204; ax[0..7] = AX01 AX02 AX10 AX11 AX12 AX20 AX21 AX22
template <class T>
int nonref(T H, int KEY, T VEL, T VELS, T VELP, T DT, T OMG, T WB, T THPP, T THSS, T ax[8]) {
  double a[9];
  // a[] in the order a00 a01 a02 a10 a11 a12 a20 a21 a22
  auto from_dp = [&](bool single) {
    const int idx[8] = {1, 2, 3, 4, 5, 6, 7, 8};
    for (int k = 0; k < 8; ++k) ax[k] = single ? (T)(float)a[idx[k]] : (T)a[idx[k]];
  };
  switch (KEY) {
    case 0:
      for (int k = 0; k < 8; ++k) ax[k] = T(0);
      return FDP_OK;
    case 1:
      higdon_fd<T>(WB, VELP, VELS, DT, H, a);
      from_dp(false);
      return FDP_OK;
    case 2: {
      const T TMP = -DT * VEL / H;
      ax[0] = T(0); ax[1] = T(0); ax[2] = T(1) + TMP; ax[3] = T(1) - TMP;
      ax[4] = T(0); ax[5] = T(0); ax[6] = -T(1) - TMP; ax[7] = TMP;
      return FDP_OK;
    }
    case 3:
    case 9: {
      // REAL(aa) without a kind is default real (nonref.F90:114-121)
      const double gplus = (double)THPP, gminus = (double)THSS;
      const double dtaux = (double)(OMG * DT);
      const double haux = (double)(OMG / (KEY == 3 ? VEL : VELS) * H);
      opt_abs_bc(gplus, gminus, dtaux, haux, a);
      from_dp(true);
      return FDP_OK;
    }
    case 4: {
      const T TMP1 = (DT - H / VEL) / (DT + H / VEL);
      const T TMP2 = T(2) * H / VEL / (DT + H / VEL);
      ax[0] = TMP1; ax[1] = T(0); ax[2] = TMP2; ax[3] = TMP2;
      ax[4] = T(0); ax[5] = TMP1; ax[6] = -T(1); ax[7] = T(0);
      return FDP_OK;
    }
    case 5: {
      const T TMP1 = VEL * DT / H;
      ax[0] = -(T(1) - TMP1) / (T(1) + TMP1); ax[1] = T(0); ax[2] = (T(1) - TMP1) / (T(1) + TMP1); ax[3] = T(1);
      ax[4] = T(0); ax[5] = T(0); ax[6] = T(0); ax[7] = T(0);
      return FDP_OK;
    }
    case 6:
      higce_fd<T>(WB, VELP, VELS, DT, H, a);
      from_dp(false);
      return FDP_OK;
    case 7:
      higce2_fd<T>(WB, VEL, VEL, DT, H, a);
      from_dp(false);
      return FDP_OK;
    case 8:
      higce2_fd<T>(WB, VELS, VELP, DT, H, a);
      from_dp(false);
      return FDP_OK;
    default:
      // SELECT CASE without a match leaves the outputs undefined in the
      // reference; an unknown key is rejected here
      return FDP_ERR_ARG;
  }
}

template <class T>
int nr_t(int MX, int MZ, int TPML, int KTBO, T DT, T H, T OMG, T WB, T THPP, T THSS, const int32_t* jm, int jmnum,
         const T* tab, T* ab) {
  const int PMLL = 1 - TPML, NX = MX + 2 * TPML;
  (void)MX;
  const int J1 = jm[(size_t)(PMLL - PMLL) + (size_t)MZ * NX];  // JM(X_MIN, MZ)
  if (J1 < 1 || J1 > jmnum) return FDP_ERR_ARG;
  T vpf, vps, vs;
  vel_x<T>(tab + (size_t)(J1 - 1) * 24, H, DT, vpf, vps, vs);
  int rc = nonref<T>(H, KTBO, vpf, vs, vpf, DT, OMG, WB, THPP, THSS, ab);
  if (rc != FDP_OK) return rc;
  return nonref<T>(H, KTBO, vs, vs, vpf, DT, OMG, WB, THPP, THSS, ab + 8);
}

// open_sr_file.F90:121-226
template <class T> void spline(const std::vector<T>& x, const std::vector<T>& y, T yp1, T ypn, std::vector<T>& y2) {
  const int n = (int)x.size();
  std::vector<T> a(n + 1), b(n + 1), c(n + 1), r(n + 1);  // 1-based
  auto X = [&](int i) { return x[i - 1]; };
  auto Y = [&](int i) { return y[i - 1]; };
  for (int i = 1; i <= n - 1; ++i) c[i] = X(i + 1) - X(i);
  for (int i = 1; i <= n - 1; ++i) r[i] = T(6) * ((Y(i + 1) - Y(i)) / c[i]);
  {
    std::vector<T> rold(r);
    for (int i = 2; i <= n - 1; ++i) r[i] = rold[i] - rold[i - 1];
  }
  for (int i = 2; i <= n - 1; ++i) a[i] = c[i - 1];
  for (int i = 2; i <= n - 1; ++i) b[i] = T(2) * (c[i] + a[i]);
  b[1] = T(1);
  b[n] = T(1);
  if (yp1 > (T)0.99e30f) { r[1] = T(0); c[1] = T(0); }
  else { r[1] = (T(3) / (X(2) - X(1))) * ((Y(2) - Y(1)) / (X(2) - X(1)) - yp1); c[1] = T(0.5); }
  if (ypn > (T)0.99e30f) { r[n] = T(0); a[n] = T(0); }
  else { r[n] = (-T(3) / (X(n) - X(n - 1))) * ((Y(n) - Y(n - 1)) / (X(n) - X(n - 1)) - ypn); a[n] = T(0.5); }
  // tridag(a(2:n), b(1:n), c(1:n-1), r(1:n), y2(1:n))
  std::vector<T> gam(n + 1), u(n + 1);
  T bet = b[1];
  u[1] = r[1] / bet;
  for (int j = 2; j <= n; ++j) {
    gam[j] = c[j - 1] / bet;
    bet = b[j] - a[j] * gam[j];
    u[j] = (r[j] - a[j] * u[j - 1]) / bet;
  }
  for (int j = n - 1; j >= 1; --j) u[j] = u[j] - gam[j + 1] * u[j + 1];
  y2.assign(n, T(0));
  for (int i = 1; i <= n; ++i) y2[i - 1] = u[i];
}

template <class T> int locate(const std::vector<T>& xx, T x) {
  const int n = (int)xx.size();
  const bool ascnd = xx[n - 1] >= xx[0];
  int jl = 0, ju = n + 1;
  while (ju - jl > 1) {
    const int jm = (ju + jl) / 2;
    if (ascnd == (x >= xx[jm - 1])) jl = jm; else ju = jm;
  }
  if (x == xx[0]) return 1;
  if (x == xx[n - 1]) return n - 1;
  return jl;
}

template <class T> T splint(const std::vector<T>& xa, const std::vector<T>& ya, const std::vector<T>& y2a, T x) {
  const int n = (int)xa.size();
  const int klo = std::max(std::min(locate(xa, x), n - 1), 1);
  const int khi = klo + 1;
  const T h = xa[khi - 1] - xa[klo - 1];
  const T a = (xa[khi - 1] - x) / h;
  const T b = (x - xa[klo - 1]) / h;
  return a * ya[klo - 1] + b * ya[khi - 1] + ((a * a * a - a) * y2a[klo - 1] + (b * b * b - b) * y2a[khi - 1]) * (h * h) / T(6);
}

template <class T>
int source_t(int nstf, const T* time, const T* stf, int MT2, T DT, T H, int KEY_SOUR, T QR, T* out) {
  if (nstf < 1) return FDP_ERR_ARG;
  for (int i = 0; i < 2 * MT2; ++i) out[i] = T(0);
  const int NSTFS = nstf + 1;
  std::vector<T> TIME(time, time + nstf), STF(stf, stf + nstf), STF2;
  TIME.push_back((T)MT2 * DT);
  STF.push_back(STF[NSTFS - 2]);
  for (int k = 1; k < NSTFS; ++k)
    if (TIME[k] == TIME[k - 1]) return FDP_ERR_ARG;  // splint would STOP (open_sr_file.F90:191)
  spline<T>(TIME, STF, T(0), T(0), STF2);
  for (int I = 1; I <= MT2; ++I) {
    const T t = (T)(I - 1) * DT;
    if (t > TIME[NSTFS - 2]) break;
    T s1 = splint<T>(TIME, STF, STF2, t), s2;
    switch (KEY_SOUR) {
      case 0: s2 = QR * s1 / (H * H); s1 = (T(1) - QR) * s1 / (H * H); break;
      case 1: s2 = T(0); s1 = s1 / (H * H); break;
      case 2: s2 = s1 / (H * H); s1 = QR * s1 / (H * H); break;
      case 3: s2 = s1 / (H * H); s1 = T(0); break;
      default: s2 = T(0); break;  // no CASE matches: SOURTF_A(1,I) stays unscaled, (2,I) stays 0
    }
    out[2 * (size_t)(I - 1)] = s1;
    out[2 * (size_t)(I - 1) + 1] = s2;
  }
  return FDP_OK;
}

}  // namespace

extern "C" {

int fdp_prep_velocities(int32_t prec, double sig1, double p, double ainv, double mu, double rel1, double rel2,
                        double rel3, double* vpf, double* vps, double* vs) {
  if (!vpf || !vps || !vs) return FDP_ERR_ARG;
  if (prec == FDP_F64) {
    double a, b, c;
    calcul_velocity<double>(sig1, p, ainv, mu, rel1, rel2, rel3, a, b, c);
    *vpf = a; *vps = b; *vs = c;
  } else {
    float a, b, c;
    calcul_velocity<float>((float)sig1, (float)p, (float)ainv, (float)mu, (float)rel1, (float)rel2, (float)rel3, a, b, c);
    *vpf = a; *vps = b; *vs = c;
  }
  return FDP_OK;
}

int fdp_prep_scale_table(int32_t prec, int32_t jmnum, double dt, double h, void* table24) {
  if (!table24 || jmnum < 1) return FDP_ERR_ARG;
  auto body = [&](auto* t, auto DT, auto H) {
    for (int j = 0; j < jmnum; ++j) {
      auto* r = t + (size_t)j * 24;
      // read_model_par.F90:63-74
      r[R1U] = DT * r[R1U] / H; r[R2U] = DT * r[R2U]; r[R3U] = DT * r[R3U] / H;
      r[R1W] = DT * r[R1W] / H; r[R2W] = DT * r[R2W]; r[R3W] = DT * r[R3W] / H;
      r[R1QX] = DT * r[R1QX] / H; r[R2QX] = DT * r[R2QX] / H; r[R3QX] = DT * r[R3QX];
      r[R1QZ] = DT * r[R1QZ] / H; r[R2QZ] = DT * r[R2QZ] / H; r[R3QZ] = DT * r[R3QZ];
    }
  };
  if (prec == FDP_F64) body((double*)table24, dt, h);
  else body((float*)table24, (float)dt, (float)h);
  return FDP_OK;
}

int fdp_prep_expand_jm(int32_t mx, int32_t mz, int32_t tpml, int32_t si, const int32_t* rows, int32_t* out) {
  if (!rows || !out || mx < 1 || mz < 4 || tpml < 0) return FDP_ERR_ARG;
  const int PMLL = 1 - tpml, PMLXH = mx + tpml, PMLZH = mz + tpml, NX = PMLXH - PMLL + 1;
  auto J = [&](int I, int L) -> int32_t& { return out[(size_t)(I - PMLL) + (size_t)L * NX]; };
  const int Lfirst = si ? 2 : 0;
  for (int L = Lfirst; L <= mz; ++L) {
    const int32_t* r = rows + (size_t)(L - Lfirst) * mx;
    for (int I = 1; I <= mx; ++I) J(I, L) = r[I - 1];
    for (int j = 0; j <= tpml; ++j) { J(1 - j, L) = J(1, L); J(mx + j, L) = J(mx, L); }
  }
  if (si) {
    // read_model.F90:64-65, final state after the loop (MZ >= 4)
    for (int I = PMLL; I <= PMLXH; ++I) { J(I, 1) = J(I, 2); J(I, 0) = J(I, 3); }
  }
  for (int L = mz + 1; L <= PMLZH; ++L)
    for (int I = PMLL; I <= PMLXH; ++I) J(I, L) = J(I, mz);
  return FDP_OK;
}

int fdp_prep_pml(int32_t prec, int32_t mx, int32_t mz, int32_t tpml, int32_t ktbo, double r, double tau, double pow_,
                 double sf, double wc, double dt, double h, const int32_t* jm, int32_t jmnum, const void* table24,
                 void* const* prof) {
  if (!jm || !table24 || !prof || mx < 1 || mz < 1 || tpml < 0) return FDP_ERR_ARG;
  for (int k = 0; k < 24; ++k) if (!prof[k]) return FDP_ERR_ARG;
  if (prec == FDP_F64)
    return pml_t<double>(mx, mz, tpml, ktbo, r, tau, pow_, sf, wc, dt, h, jm, jmnum, (const double*)table24, prof);
  return pml_t<float>(mx, mz, tpml, ktbo, (float)r, (float)tau, (float)pow_, (float)sf, (float)wc, (float)dt,
                      (float)h, jm, jmnum, (const float*)table24, prof);
}

int fdp_prep_bottom_nr(int32_t prec, int32_t mx, int32_t mz, int32_t tpml, int32_t ktbo, double dt, double h,
                       double omg, double wb, double thpple, double thssle, const int32_t* jm, int32_t jmnum,
                       const void* table24, void* ab16) {
  if (!jm || !table24 || !ab16) return FDP_ERR_ARG;
  if (prec == FDP_F64)
    return nr_t<double>(mx, mz, tpml, ktbo, dt, h, omg, wb, thpple, thssle, jm, jmnum, (const double*)table24,
                        (double*)ab16);
  return nr_t<float>(mx, mz, tpml, ktbo, (float)dt, (float)h, (float)omg, (float)wb, (float)thpple, (float)thssle, jm,
                     jmnum, (const float*)table24, (float*)ab16);
}

int fdp_prep_source(int32_t prec, int32_t nstf, const void* time, const void* stf, int32_t mt2, double dt, double h,
                    int32_t key_sour, double qr, void* sourtf) {
  if (!time || !stf || !sourtf || mt2 < 1) return FDP_ERR_ARG;
  if (prec == FDP_F64)
    return source_t<double>(nstf, (const double*)time, (const double*)stf, mt2, dt, h, key_sour, qr, (double*)sourtf);
  return source_t<float>(nstf, (const float*)time, (const float*)stf, mt2, (float)dt, (float)h, key_sour, (float)qr,
                         (float*)sourtf);
}

}  // extern "C"
