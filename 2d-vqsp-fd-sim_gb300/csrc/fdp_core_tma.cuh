// TMA-staged core kernels (FP32, Biot planes): the same cells and the same
// arithmetic as k_stress_core / k_velocity_core, with every input of a core
// tile (128 columns x 8 rows) brought into shared memory by bulk tensor
// copies (cp.async.bulk.tensor.2d) instead of per-thread loads.
//
// A persistent CTA of 256 threads (one per SM) walks the tiles of the core
// with kCStages shared-memory stages: while it computes one tile, the copies
// of the next kCStages-1 tiles are in flight.  One thread issues the 13
// copies of a tile -- the phase's 4 stencil inputs with their halo, its 4
// read-modify-write fields and its 5 medium planes -- on the stage's
// mbarrier; every thread waits for it with a bounded try_wait.  A wait that
// gives up sets the status word; the CTA then waits (bounded) for each copy
// it still has in flight and returns.  Results go out with 16-byte global
// stores.  Every copy starts on a 16-byte-aligned column (the core's first
// column and the padded pitch are multiples of 4 floats), no row is
// negative (the core starts at row 2), and boxes reaching past the array
// read zeros that no cell uses.
#pragma once

#include "fdp_stencil.cuh"

namespace fdp {

constexpr int kCTW = 4 * kBX;   // tile width (columns), 4 per thread
constexpr int kCTH = kBZ;       // tile height (rows), 1 per thread
constexpr int kCHW = kCTW + 8;  // input box width: 4 columns of halo either side
constexpr int kCHH = kCTH + 3;  // input box height with the z-stencil rows
constexpr int kCStages = 3;

// A phase's tensor maps: [0..3] stencil inputs (boxes kCHW x kCHH, or
// kCHW x kCTH for the one read on its own row only), [4..7] updated fields
// and [8..12] medium planes (boxes kCTW x kCTH).
struct CoreMaps {
  CUtensorMap m[13];
};

// first row of input box k relative to the tile's first row, and its height
//   stress:   U rows L-2..L+1, W L-1..L+2, QX L, QZ L-1..L+2
//   velocity: TXX L, TZZ L-2..L+1, TXZ L-1..L+2, PRES L-2..L+1
__host__ __device__ constexpr int core_box_row(int phase, int k) {
  return phase == 0 ? (k == 0 ? -2 : k == 2 ? 0 : -1) : (k == 0 ? 0 : k == 2 ? -1 : -2);
}
__host__ __device__ constexpr int core_box_rows(int phase, int k) {
  return (phase == 0 ? k == 2 : k == 0) ? kCTH : kCHH;
}

constexpr int kInBox = (kCHH * kCHW + 31) / 32 * 32;  // floats, 128-byte multiple
constexpr int kTileBox = kCTH * kCTW;
constexpr int kStageFloats = 4 * kInBox + 9 * kTileBox;
constexpr size_t kCoreTmaSmem = (size_t)kCStages * kStageFloats * sizeof(float) + 128;
static_assert(kCoreTmaSmem <= 227 * 1024, "stages exceed the shared memory of a CTA");
static_assert((kInBox * 4) % 128 == 0 && (kTileBox * 4) % 128 == 0, "boxes must start 128-byte aligned");

__host__ __device__ constexpr uint32_t core_stage_bytes(int phase) {
  return 4u * (uint32_t)((core_box_rows(phase, 0) + core_box_rows(phase, 1) + core_box_rows(phase, 2) +
                          core_box_rows(phase, 3)) * kCHW + 9 * kTileBox);
}

__device__ __forceinline__ V4<float> lds4(const float* s) {
  const float4 v = *reinterpret_cast<const float4*>(s);
  return {{v.x, v.y, v.z, v.w}};
}

// Issues the copies of the tile whose first cell is padded column `col`,
// padded row `row`, into stage `st`.
template <int PHASE>
__device__ __forceinline__ void core_issue(float* st, uint64_t* bar, const CoreMaps& maps, int col, int row) {
  mbar_expect_tx(bar, core_stage_bytes(PHASE));
#pragma unroll
  for (int k = 0; k < 4; ++k) tma_load_2d(st + k * kInBox, &maps.m[k], col - 4, row + core_box_row(PHASE, k), bar);
#pragma unroll
  for (int k = 0; k < 9; ++k) tma_load_2d(st + 4 * kInBox + k * kTileBox, &maps.m[4 + k], col, row, bar);
}

struct CoreTiles {
  int x0, x1, z0, z1;  // the phase's core rectangle
  int gx, n;           // tiles along x, tiles in all
};

__host__ __device__ inline CoreTiles core_tiles(const Params<float>& p, int phase) {
  CoreTiles t;
  t.x0 = phase == 0 ? p.cs_x0 : p.cv_x0; t.x1 = phase == 0 ? p.cs_x1 : p.cv_x1;
  t.z0 = phase == 0 ? p.cs_z0 : p.cv_z0; t.z1 = phase == 0 ? p.cs_z1 : p.cv_z1;
  t.gx = (t.x1 - t.x0 + kCTW - 1) / kCTW;
  t.n = t.gx * ((t.z1 - t.z0 + kCTH - 1) / kCTH);
  return t;
}

// PHASE 0: the stress core (stress_core_block's cells), 1: the velocity core.
template <int PHASE>
__global__ void __launch_bounds__(kBX * kBZ, 1) k_core_tma(const __grid_constant__ Params<float> p,
                                                            const __grid_constant__ CoreMaps maps) {
  extern __shared__ unsigned char smem_raw[];
  float* const smem = reinterpret_cast<float*>(((uintptr_t)smem_raw + 127) & ~(uintptr_t)127);
  __shared__ __align__(8) uint64_t full[kCStages];
  __shared__ int failed;
  const CoreTiles g = core_tiles(p, PHASE);
  const int tid = (int)(threadIdx.y * kBX + threadIdx.x);
  const int first = (int)blockIdx.x, step = (int)gridDim.x;
  auto issue = [&](int i) {  // the CTA's i-th tile into stage i % kCStages
    const int t = first + i * step;
    const int bx = t % g.gx, by = t / g.gx;
    core_issue<PHASE>(smem + (i % kCStages) * kStageFloats, &full[i % kCStages], maps,
                      g.x0 + kCTW * bx - p.PMLL + kPadX, g.z0 + kCTH * by + kPadZ);
  };
  const int mine = first < g.n ? (g.n - first + step - 1) / step : 0;  // tiles of this CTA
  if (tid == 0) {
    for (int s = 0; s < kCStages; ++s) mbar_init(&full[s], 1);
    failed = 0;
  }
  __syncthreads();
  if (tid == 0)
    for (int i = 0; i < kCStages && i < mine; ++i) issue(i);
  const float A = p.A, B = p.B;
  int i = 0;
  for (; i < mine; ++i) {
    const int s = i % kCStages;
    if (!mbar_wait_bounded(&full[s], (uint32_t)((i / kCStages) & 1))) failed = 1;
    __syncthreads();
    if (failed) break;
    const float* S = smem + s * kStageFloats;
    const int t = first + i * step;
    const int bx = t % g.gx, by = t / g.gx;
    const int ty = (int)threadIdx.y, c4 = 4 * (int)threadIdx.x;
    const int I0 = g.x0 + kCTW * bx + c4;
    const int L = g.z0 + kCTH * by + ty;
    // row r of input box k (r counted from the box's first row), the
    // thread's 4 columns shifted by dc
    auto in4 = [&](int k, int r, int dc) { return lds4(S + k * kInBox + r * kCHW + 4 + c4 + dc); };
    auto tile4 = [&](int k) { return lds4(S + 4 * kInBox + k * kTileBox + ty * kCTW + c4); };
    auto at = [](const V4<float>* r, int j, int d) { return r[(j + d + 4) >> 2].v[(j + d + 4) & 3]; };
    if (I0 < g.x1 && L < g.z1 && (PHASE != 0 || L != p.LIN_Z)) {
      const long long c0 = (long long)L * p.pitch + (I0 - p.PMLL);
      V4<float> bio[5];
#pragma unroll
      for (int k = 0; k < 5; ++k) bio[k] = tile4(4 + k);
      if (PHASE == 0) {
        // box rows: U from L-2, W and QZ from L-1, QX from L
        const V4<float> ur[3] = {in4(0, ty + 2, -4), in4(0, ty + 2, 0), in4(0, ty + 2, 4)};
        const V4<float> wr[3] = {in4(1, ty + 1, -4), in4(1, ty + 1, 0), in4(1, ty + 1, 4)};
        const V4<float> xr[3] = {in4(2, ty, -4), in4(2, ty, 0), in4(2, ty, 4)};
        const V4<float> um2 = in4(0, ty, 0), um1 = in4(0, ty + 1, 0), up1 = in4(0, ty + 3, 0);
        const V4<float> wm1 = in4(1, ty, 0), wp1 = in4(1, ty + 2, 0), wp2 = in4(1, ty + 3, 0);
        const V4<float> zm1 = in4(3, ty, 0), z0 = in4(3, ty + 1, 0), zp1 = in4(3, ty + 2, 0),
                        zp2 = in4(3, ty + 3, 0);
        V4<float> oxx = tile4(0), ozz = tile4(1), oxz = tile4(2), opr = tile4(3);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          auto C = [&](int k) { return core_coef<float, M_BIOT>(p, k, 0, 0, bio, 0, j); };
          // strain_uw_xz.F90:81-84
          const float exz = p.AH * (up1.v[j] - um2.v[j] + at(wr, j, 1) - at(wr, j, -2))
                          + p.BH * (ur[1].v[j] - um1.v[j] + wr[1].v[j] - at(wr, j, -1));
          // strain_uw_zz.F90:51,58-59 and strain_q_zz.F90:48,55-56
          float ezz = (p.CH * (wp1.v[j] - wr[1].v[j]));
          ezz = p.AH * (wp2.v[j] - wm1.v[j]) + p.BC * ezz;
          float qzz = (p.CH * (zp1.v[j] - z0.v[j]));
          qzz = p.AH * (zp2.v[j] - zm1.v[j]) + p.BC * qzz;
          // strain_uw_xx.F90:82-83 and strain_q_xx.F90:77-78
          const float exx = p.AH * (at(ur, j, 2) - at(ur, j, -1)) + p.BH * (at(ur, j, 1) - ur[1].v[j]);
          const float qxx = p.AH * (at(xr, j, 2) - at(xr, j, -1)) + p.BH * (at(xr, j, 1) - xr[1].v[j]);
          // stress_xz.F90:44-46 and stress_nn.F90:53-59
          const float TXZv = C(C_MU) * exz;
          oxz.v[j] = oxz.v[j] + p.DTE * TXZv;
          const float s1 = C(C_SXX1), s2 = C(C_SXX2), s3 = C(C_SXX3);
          const float z1 = C(C_SZZ1), z2 = C(C_SZZ2), z3 = C(C_SZZ3);
          const float q1 = C(C_P1), q2 = C(C_P2), q3 = C(C_P3);
          const float TXXv = s1 * exx + s2 * ezz + s3 * qxx + s3 * qzz;
          const float TZZv = z1 * exx + z2 * ezz + z3 * qxx + z3 * qzz;
          const float PRv = q1 * exx + q2 * ezz + q3 * qxx + q3 * qzz;
          oxx.v[j] = oxx.v[j] + p.DTE * TXXv;
          ozz.v[j] = ozz.v[j] + p.DTE * TZZv;
          opr.v[j] = opr.v[j] + p.DTE * PRv;
        }
        st4(p.oTXZ + c0, oxz);
        st4(p.oTXX + c0, oxx);
        st4(p.oTZZ + c0, ozz);
        st4(p.oPRES + c0, opr);
      } else {
        // box rows: TXX from L, TZZ and PRES from L-2, TXZ from L-1
        const V4<float> xxr[3] = {in4(0, ty, -4), in4(0, ty, 0), in4(0, ty, 4)};
        const V4<float> prr[3] = {in4(3, ty + 2, -4), in4(3, ty + 2, 0), in4(3, ty + 2, 4)};
        const V4<float> xzr[3] = {in4(2, ty + 1, -4), in4(2, ty + 1, 0), in4(2, ty + 1, 4)};
        const V4<float> prm2 = in4(3, ty, 0), prm1 = in4(3, ty + 1, 0), prp1 = in4(3, ty + 3, 0);
        const V4<float> xzm1 = in4(2, ty, 0), xzp1 = in4(2, ty + 2, 0), xzp2 = in4(2, ty + 3, 0);
        const V4<float> zzm2 = in4(1, ty, 0), zzm1 = in4(1, ty + 1, 0), zz0 = in4(1, ty + 2, 0),
                        zzp1 = in4(1, ty + 3, 0);
        V4<float> oqx = tile4(0), oum = tile4(1), oqz = tile4(2), owm = tile4(3);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          auto C = [&](int k) { return core_coef<float, M_BIOT>(p, k, 0, 0, bio, 5, j); };
          const float pr0 = prr[1].v[j];
          {
            // inh_qx_int.F90:44-52 and inh_v_uv_int.F90:45-54
            const float E = C(C_EQX), Cu = C(C_CU);
            const float R1 = C(C_R1QX), R2 = C(C_R2QX), R1u = C(C_R1U), R3u = C(C_R3U);
            const float qx0 = oqx.v[j], u0 = oum.v[j];
            const float Xs = A * (at(xxr, j, 1) - at(xxr, j, -2) + xzp2.v[j] - xzm1.v[j])
                           + B * (xxr[1].v[j] - at(xxr, j, -1) + xzp1.v[j] - xzr[1].v[j]);
            const float Pp = A * (at(prr, j, 1) - at(prr, j, -2)) + B * (pr0 - at(prr, j, -1));
            oqx.v[j] = E * qx0 - R1 * Xs - R2 * Pp;
            oum.v[j] = u0 + Cu * qx0 + R1u * Xs + R3u * Pp;
          }
          {
            // inh_qz_int.F90:45-53 and inh_v_w_int.F90:47-56
            const float E = C(C_EQZ), Cw = C(C_CW);
            const float R1 = C(C_R1QZ), R2 = C(C_R2QZ), R1w = C(C_R1W), R3w = C(C_R3W);
            const float qz0 = oqz.v[j], w0 = owm.v[j];
            const float Xs = A * (zzp1.v[j] - zzm2.v[j] + at(xzr, j, 2) - at(xzr, j, -1))
                           + B * (zz0.v[j] - zzm1.v[j] + at(xzr, j, 1) - xzr[1].v[j]);
            const float Pp = A * (prp1.v[j] - prm2.v[j]) + B * (pr0 - prm1.v[j]);
            oqz.v[j] = E * qz0 - R1 * Xs - R2 * Pp;
            owm.v[j] = w0 + Cw * qz0 + R1w * Xs + R3w * Pp;
          }
        }
        st4(p.oQX + c0, oqx);
        st4(p.oUM + c0, oum);
        st4(p.oQZ + c0, oqz);
        st4(p.oWM + c0, owm);
      }
    }
    __syncthreads();  // every thread is done with stage s
    if (tid == 0 && i + kCStages < mine) issue(i + kCStages);
  }
  if (i < mine && tid == 0) {
    // a wait gave up at tile i: report it, then let the copies this CTA
    // still has in flight (tiles i .. i+kCStages-1) land before its shared
    // memory is released
    atomicOr(p.err, 2);
    for (int j = i; j < i + kCStages && j < mine; ++j)
      mbar_wait_bounded(&full[j % kCStages], (uint32_t)((j / kCStages) & 1));
  }
}

}  // namespace fdp
