// A whole time level of the deep interior in one pass (the "march" kernel).
//
// A level is the stress phase (time_loop.F90:93-124) and then the velocity
// phase (time_loop.F90:133-179).  In the interior both are the 4th-order
// stencils of the core kernels, and a cell's new velocities need the new
// stresses only within two cells of it.  So a CTA of R warps (R = 4, 6 or
// 8) owns a strip of 30 four-cell vectors (120 columns) and marches down a
// range of its rows in bands of R rows.  Step k of a range computes, after
// one block barrier, the new velocities of band k-1 (each warp one row,
// from the new stresses of the rows two above to two below it, kept in a
// shared-memory ring of 2R+4 rows) and the new stresses of band k (each
// warp one row, for the strip's vectors and one halo vector either side:
// lanes 0 and 31), which go into the ring.  A cell's stencils read the old
// wavefield (one buffer of each pair) and write the new values to the
// other, so no CTA reads what another writes during the launch.
//
// Inputs arrive by bulk tensor copies (cp.async.bulk.tensor.2d), one box of
// 128 columns by R rows per array: the old velocities into a ring of 4R
// rows (the 3R+4 a step reads and the next band's R), the old stresses and
// the five stress planes of band k and the five velocity planes of band k-1
// into one of two stages.  One thread issues the next step's copies as a
// step starts, so they are in flight while the step computes; every thread
// waits for its step's copies on the stage's mbarrier with a bounded
// try_wait, and a wait that gives up sets the status word, lets the copies
// in flight land (bounded again) and returns.
//
// Per cell the pass reads the old velocities and stresses and the ten
// coefficient planes and writes the new velocities and stresses: 26 values
// (104 bytes in FP32), where the two phases as separate passes read the new
// stresses and the old velocities a second time (136 bytes).
//
// The region F the kernel updates, [fx0, fx1) x [fz0, fz1), is chosen on
// the host so that every stencil the kernel evaluates, including the new
// stresses of the halo cells two columns and two rows around F, is the
// interior one; the frame kernels update every other cell.  The kernel
// writes the new velocities of all of F, and the new stresses of F less a
// band of one vector and two rows along its edges: the frame kernel's
// velocity cells next to F read the new stresses there, and the frame
// kernels (on another stream) write them instead, so the launches need no
// ordering between them.  The stress update of the source cell (LIN_X,
// LIN_Z) adds the source term of stress_lin_nn.F90:58-63.
//
// The CTAs take contiguous ranges of the rows of all strips taken as one
// sequence (one CTA per SM, two with bands of four rows): the same number
// of CTAs on every strip, or, with more strips than CTAs, whole strips per
// CTA, so that the CTAs march down the same rows together.  A CTA whose
// range crosses into the next strip starts again there.  FP32; a medium
// held as the ten Biot planes has them staged with the stresses, any other
// reaches its coefficients through the kernels' lookup (a material index
// read per cell into a cached table, or constants folded into the
// parameters).
#pragma once

#include "fdp_core_tma.cuh"

namespace fdp {

constexpr int kMarchVec = 30;  // vectors a strip updates (lanes 1..30)
constexpr int kMarchW = 128;   // box width: the strip's 32 vectors

// Boxes of a stage: the old stresses (4) and, for a medium held as the ten
// Biot planes, the five stress planes and the five velocity planes; other
// media reach their coefficients through the kernels' coefficient lookup
// (a material index into a cached table, or constants).
__host__ __device__ constexpr int march_boxes(int mode) { return mode == M_BIOT ? 14 : 4; }

// Sizes of a CTA of R warps marching bands of R rows (R = 4, 6 or 8) with
// stages of NB boxes.  A step reads 3R+4 rows of the velocity ring while
// the next band's R rows arrive, and 2R+4 rows of the stress ring (R
// written, R+4 read).
template <int R, int NB> struct MarchShape {
  static constexpr int kThreads = 32 * R;
  static constexpr int kVRows = 4 * R;      // velocity ring rows (slots of R)
  static constexpr int kSRows = 2 * R + 4;  // stress ring rows
  static constexpr int kBox = R * kMarchW;  // floats per box
  static constexpr int kVRing = 4 * kVRows * kMarchW;
  static constexpr int kStage = NB * kBox;
  static constexpr int kSRing = 4 * kSRows * kMarchW;
  static constexpr size_t kSmem = (size_t)(kVRing + 2 * kStage + kSRing) * sizeof(float) + 128;
  // CTAs of this shape that fit an SM's 228 KB (1 KB reserved per CTA)
  static constexpr int kCtasPerSm = kSmem <= 74 * 1024 ? 3 : kSmem <= 113 * 1024 ? 2 : 1;
  static_assert(kSmem <= 227 * 1024, "march stages exceed the shared memory of a CTA");
  static_assert(R >= 4, "a band's stencils reach four rows back");
};
template <int MODE, int R> using MarchShapeOf = MarchShape<R, march_boxes(MODE)>;

// Tensor maps (boxes of 128 columns by R rows): the eight wavefield arrays
// a level reads (UM WM QX QZ TXX TZZ TXZ PRES) and the ten Biot planes.
struct MarchMaps {
  CUtensorMap f[8];
  CUtensorMap pl[10];
};

// The launch's work: F, where the new stresses are written, the strips of
// kMarchVec vectors across F, and the rows of all strips as one sequence.
struct MarchGrid {
  int fx0, fx1, fz0, fz1;  // F
  int sx0, sx1, sz0, sz1;  // where the kernel writes the new stresses
  int nstrips, nvec;       // strips, vectors across F
  long long total;         // nstrips * (fz1 - fz0)
  long long span;          // rows of a CTA's range (whole strips), or 0: total split evenly
};

// A step of a CTA: strip, the velocity rows [vlo, vhi) of its segment and
// its index k there.  Band k's stresses are rows [vlo-2+Rk, vlo-2+R(k+1))
// and its velocities the rows two above those; step k computes the
// stresses of band k and the velocities of band k-1.  strip < 0: past the
// CTA's range.
struct MarchBand {
  int strip, vlo, vhi, k;
};

// 16 bytes of shared memory (a 16-byte-aligned shared address)
__device__ __forceinline__ V4<float> lds4s(const float* s) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"((uint32_t)__cvta_generic_to_shared(s)));
  return {{v.x, v.y, v.z, v.w}};
}
__device__ __forceinline__ void sts4s(float* s, const V4<float>& v) {
  asm volatile("st.shared.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"((uint32_t)__cvta_generic_to_shared(s)), "f"(v.v[0]),
               "f"(v.v[1]), "f"(v.v[2]), "f"(v.v[3])
               : "memory");
}

template <int MODE, int R>
__global__ void __launch_bounds__(MarchShapeOf<MODE, R>::kThreads, MarchShapeOf<MODE, R>::kCtasPerSm)
    k_march(const __grid_constant__ Params<float> p, const __grid_constant__ MarchMaps maps, const MarchGrid g,
            int it_off) {
  using Sh = MarchShapeOf<MODE, R>;
  constexpr bool kPlanes = MODE == M_BIOT;  // coefficient planes staged with the stresses
  extern __shared__ unsigned char march_raw[];
  float* const vring = reinterpret_cast<float*>(((uintptr_t)march_raw + 127) & ~(uintptr_t)127);
  float* const stages = vring + Sh::kVRing;
  float* const sring = stages + 2 * Sh::kStage;
  __shared__ __align__(8) uint64_t full[2];
  __shared__ int failed;
  const int tid = (int)threadIdx.x, lane = tid & 31, warp = tid >> 5;
  // the CTA's rows [lo, hi) of the sequence of all strips' rows (H per strip)
  const int H = g.fz1 - g.fz0;
  const long long lo = g.span ? blockIdx.x * g.span : (long long)blockIdx.x * g.total / gridDim.x;
  const long long hi = g.span ? (lo + g.span < g.total ? lo + g.span : g.total)
                              : (long long)(blockIdx.x + 1) * g.total / gridDim.x;
  auto seg_end = [&](int strip) {  // the end of strip `strip`'s rows in the range
    const long long e = (long long)(strip + 1) * H;
    return g.fz0 + (int)((e <= hi ? e : hi) - (long long)strip * H);
  };
  // bands of a segment: their stresses reach two rows past its last velocity row
  auto nbands = [&](const MarchBand& b) { return (b.vhi - b.vlo + 4 + R - 1) / R; };
  // steps k = 0 .. nbands of a segment, then the next segment's
  auto next = [&](const MarchBand& b) -> MarchBand {
    if (b.strip < 0) return b;
    if (b.k < nbands(b)) return {b.strip, b.vlo, b.vhi, b.k + 1};
    const int s = b.strip + 1;
    if ((long long)s * H >= hi) return {-1, 0, 0, 0};
    return {s, g.fz0, seg_end(s), 0};
  };
  if (tid == 0) {
    mbar_init(&full[0], 1);
    mbar_init(&full[1], 1);
    failed = 0;
  }
  __syncthreads();
  if (lo >= hi) return;

  // the copies of step b (the CTA's j-th) on barrier j % 2: band k's new
  // velocity rows into the ring, its old stresses and stress planes into
  // the stage (k < nbands), and band k-1's velocity planes (k >= 1).  The
  // ring slots rotate with the CTA's steps, across segments too: step j's
  // band goes to slot (j+1) % 4 and a segment's first rows, [vlo-R, vlo),
  // to slot j % 4, so a ring row of step j's segment is at
  // (4R + R*j + R - 2 + y - r) % 4R for grid row y (r its first stress row)
  auto issue = [&](const MarchBand& b, int j) {
    uint64_t* bar = &full[j & 1];
    float* st = stages + (j & 1) * Sh::kStage;
    const int x = g.fx0 + 4 * kMarchVec * b.strip - 4 - p.PMLL + kPadX;  // padded column of the box
    const int r = b.vlo - 2 + R * b.k;                                      // band k's first stress row
    const bool s_ = b.k < nbands(b), v_ = b.k >= 1;
    const int boxes = (s_ ? (b.k == 0 ? 12 : 8) + (kPlanes ? 5 : 0) : 0) + (v_ && kPlanes ? 5 : 0);
    mbar_expect_tx(bar, (uint32_t)(boxes * Sh::kBox * sizeof(float)));
    if (s_) {
      const int slot = ((j + 1) & 3) * R, pro = (j & 3) * R;
#pragma unroll
      for (int f = 0; f < 4; ++f) {
        float* fr = vring + f * Sh::kVRows * kMarchW;
        tma_load_2d(fr + slot * kMarchW, &maps.f[f], x, r + 2 + kPadZ, bar);
        if (b.k == 0) tma_load_2d(fr + pro * kMarchW, &maps.f[f], x, b.vlo - R + kPadZ, bar);
      }
#pragma unroll
      for (int f = 0; f < 4; ++f) tma_load_2d(st + f * Sh::kBox, &maps.f[4 + f], x, r + kPadZ, bar);
      if constexpr (kPlanes) {
#pragma unroll
        for (int s = 0; s < 5; ++s) tma_load_2d(st + (4 + s) * Sh::kBox, &maps.pl[s], x, r + kPadZ, bar);
      }
    }
    if (v_ && kPlanes) {
      // band k-1's velocity rows [r-R-2, r-2)
#pragma unroll
      for (int s = 0; s < 5; ++s) tma_load_2d(st + (9 + s) * Sh::kBox, &maps.pl[5 + s], x, r - R - 2 + kPadZ, bar);
    }
  };
  const long long P = p.pitch;
  const int it = *p.it_base + it_off;
  float srcS, srcF;
  {
    const float SOURS = p.STF[2 * (it - 1)], SOURF = p.STF[2 * (it - 1) + 1];
    const float SOURSP = it > 1 ? p.STF[2 * (it - 2)] : 0.f;
    const float SOURFP = it > 1 ? p.STF[2 * (it - 2) + 1] : 0.f;
    srcS = ((SOURS - SOURSP) / p.DT);
    srcF = ((SOURF - SOURFP) / p.DT);
  }
  const int lm = lane > 0 ? lane - 1 : 0, lp = lane < 31 ? lane + 1 : 31;  // x-neighbour vectors (clamped)
  auto wrapv = [](int r) { return r >= Sh::kVRows ? r - Sh::kVRows : (r < 0 ? r + Sh::kVRows : r); };
  auto wraps = [](int r) { return r >= Sh::kSRows ? r - Sh::kSRows : (r < 0 ? r + Sh::kSRows : r); };

  const int strip0 = (int)(lo / H);
  MarchBand b = {strip0, g.fz0 + (int)(lo - (long long)strip0 * H), seg_end(strip0), 0};
  int vk = 0, sk = 0;  // R*j modulo the ring sizes
  int j = 0;
  bool issued = false;  // step j+1's copies are in flight
  for (; b.strip >= 0; ++j) {
    // the next step's copies go out as this one starts: a new segment's
    // first step follows the old segment's last, which computes velocities
    // only and reads the ring slots (j-1) % 4 and j % 4, while the new
    // segment's copies go to slots (j+1) % 4 and (j+2) % 4
    const MarchBand nb = next(b);
    if (tid == 0) {
      if (j == 0) issue(b, 0);
      if (nb.strip >= 0) issue(nb, j + 1);
    }
    issued = nb.strip >= 0;
    const int nbk = nbands(b);
    const float* S = stages + (j & 1) * Sh::kStage;
    const int v = kMarchVec * b.strip + lane - 1;                  // the lane's vector of F
    const int I0 = g.fx0 + 4 * v;                                  // its first column
    const bool sok = v <= g.nvec;                                  // new stresses here (halo included)
    const bool own = lane >= 1 && lane <= kMarchVec && v < g.nvec;  // a vector of F this CTA updates

    // ---- new velocities of band k-1's row Lv from the stress ring (rows
    // Lv-2..Lv+2; stress row r + w of step j's band at ring row
    // (R*j + w) % kSRows) and the old velocities
    const int Lv = b.vlo - 4 + R * (b.k - 1) + warp;
    const bool vel = b.k >= 1 && own && Lv >= b.vlo && Lv < b.vhi;
    VelocityCoreIn<float> va;
    V4<float> oum, owm, oqx, oqz;
    if (vel) {
      const int sb = sk - R - 2 + warp;
      auto srow = [&](int f, int d) { return sring + (f * Sh::kSRows + wraps(sb + d)) * kMarchW; };
      va.xxr[0] = lds4s(srow(1, 0) + 4 * lm); va.xxr[1] = lds4s(srow(1, 0) + 4 * lane);
      va.xxr[2] = lds4s(srow(1, 0) + 4 * lp);
      va.prr[0] = lds4s(srow(3, 0) + 4 * lm); va.prr[1] = lds4s(srow(3, 0) + 4 * lane);
      va.prr[2] = lds4s(srow(3, 0) + 4 * lp);
      va.xzr[0] = lds4s(srow(0, 0) + 4 * lm); va.xzr[1] = lds4s(srow(0, 0) + 4 * lane);
      va.xzr[2] = lds4s(srow(0, 0) + 4 * lp);
      va.prm2 = lds4s(srow(3, -2) + 4 * lane); va.prm1 = lds4s(srow(3, -1) + 4 * lane);
      va.prp1 = lds4s(srow(3, 1) + 4 * lane);
      va.xzm1 = lds4s(srow(0, -1) + 4 * lane); va.xzp1 = lds4s(srow(0, 1) + 4 * lane);
      va.xzp2 = lds4s(srow(0, 2) + 4 * lane);
      va.zzm2 = lds4s(srow(2, -2) + 4 * lane); va.zzm1 = lds4s(srow(2, -1) + 4 * lane);
      va.zz0 = lds4s(srow(2, 0) + 4 * lane); va.zzp1 = lds4s(srow(2, 1) + 4 * lane);
      const int vr = wrapv(vk - 4 + warp);
      oum = lds4s(vring + (0 * Sh::kVRows + vr) * kMarchW + 4 * lane);
      owm = lds4s(vring + (1 * Sh::kVRows + vr) * kMarchW + 4 * lane);
      oqx = lds4s(vring + (2 * Sh::kVRows + vr) * kMarchW + 4 * lane);
      oqz = lds4s(vring + (3 * Sh::kVRows + vr) * kMarchW + 4 * lane);
    }
    // this step's copies (issued a step ahead): a wait that gives up marks
    // the CTA failed; its values are then garbage and it stops after the step
    if (!mbar_wait_bounded(&full[j & 1], (uint32_t)((j >> 1) & 1))) failed = 1;
    if (vel) {
      V4<float> bio[5];
      if constexpr (kPlanes) {
        const float* prow = S + 9 * Sh::kBox + warp * kMarchW + 4 * lane;
#pragma unroll
        for (int s = 0; s < 5; ++s) bio[s] = lds4s(prow + s * Sh::kBox);
      }
      const long long c0 = (long long)Lv * P + (I0 - p.PMLL);
      velocity_core_math<float, MODE>(p, c0, va, bio, oqx, oum, oqz, owm);
      st4(p.oQX + c0, oqx);
      st4(p.oUM + c0, oum);
      st4(p.oQZ + c0, oqz);
      st4(p.oWM + c0, owm);
    }

    // ---- new stresses of band k's row Ls for the strip's 32 vectors
    const int Ls = b.vlo - 2 + R * b.k + warp;
    if (b.k < nbk && sok) {
      const int vb = vk + R - 2 + warp;
      auto vrow = [&](int f, int d) { return vring + (f * Sh::kVRows + wrapv(vb + d)) * kMarchW; };
      StressCoreIn<float> a;
      a.ur[0] = lds4s(vrow(0, 0) + 4 * lm); a.ur[1] = lds4s(vrow(0, 0) + 4 * lane); a.ur[2] = lds4s(vrow(0, 0) + 4 * lp);
      a.wr[0] = lds4s(vrow(1, 0) + 4 * lm); a.wr[1] = lds4s(vrow(1, 0) + 4 * lane); a.wr[2] = lds4s(vrow(1, 0) + 4 * lp);
      a.xr[0] = lds4s(vrow(2, 0) + 4 * lm); a.xr[1] = lds4s(vrow(2, 0) + 4 * lane); a.xr[2] = lds4s(vrow(2, 0) + 4 * lp);
      a.um2 = lds4s(vrow(0, -2) + 4 * lane); a.um1 = lds4s(vrow(0, -1) + 4 * lane);
      a.up1 = lds4s(vrow(0, 1) + 4 * lane);
      a.wm1 = lds4s(vrow(1, -1) + 4 * lane); a.wp1 = lds4s(vrow(1, 1) + 4 * lane);
      a.wp2 = lds4s(vrow(1, 2) + 4 * lane);
      a.zm1 = lds4s(vrow(3, -1) + 4 * lane); a.z0 = lds4s(vrow(3, 0) + 4 * lane);
      a.zp1 = lds4s(vrow(3, 1) + 4 * lane); a.zp2 = lds4s(vrow(3, 2) + 4 * lane);
      const float* srow0 = S + warp * kMarchW + 4 * lane;
      // stage boxes 0..3: TXX TZZ TXZ PRES
      V4<float> oxx = lds4s(srow0), ozz = lds4s(srow0 + Sh::kBox), oxz = lds4s(srow0 + 2 * Sh::kBox),
                opr = lds4s(srow0 + 3 * Sh::kBox);
      V4<float> bio[5];
      if constexpr (kPlanes) {
#pragma unroll
        for (int s = 0; s < 5; ++s) bio[s] = lds4s(srow0 + (4 + s) * Sh::kBox);
      }
      const long long c0 = (long long)Ls * P + (I0 - p.PMLL);
      const int src_j = (Ls == p.LIN_Z && p.LIN_X >= I0 && p.LIN_X < I0 + 4) ? p.LIN_X - I0 : -1;
      stress_core_math<float, MODE>(p, c0, a, bio, oxz, oxx, ozz, opr, src_j, srcS, srcF);
      float* sw = sring + wraps(sk + warp) * kMarchW + 4 * lane;
      sts4s(sw, oxz);
      sts4s(sw + Sh::kSRows * kMarchW, oxx);
      sts4s(sw + 2 * Sh::kSRows * kMarchW, ozz);
      sts4s(sw + 3 * Sh::kSRows * kMarchW, opr);
      if (own && I0 >= g.sx0 && I0 < g.sx1 && Ls >= b.vlo && Ls < b.vhi && Ls >= g.sz0 && Ls < g.sz1) {
        st4(p.oTXZ + c0, oxz);
        st4(p.oTXX + c0, oxx);
        st4(p.oTZZ + c0, ozz);
        st4(p.oPRES + c0, opr);
      }
    }
    __syncthreads();  // the stage, the new stresses and the ring rows later copies overwrite
    if (failed) {
      if (tid == 0) atomicOr(p.err, 1);
      break;
    }
    vk = vk + R >= Sh::kVRows ? vk + R - Sh::kVRows : vk + R;
    sk = sk + R >= Sh::kSRows ? sk + R - Sh::kSRows : sk + R;
    b = nb;
  }
  // after a wait that gave up, let the copies still in flight (this step's
  // and the next one's) land before the CTA exits (bounded)
  if (failed && tid == 0)
    for (int q = j; q <= j + (issued ? 1 : 0); ++q) mbar_wait_bounded(&full[q & 1], (uint32_t)((q >> 1) & 1));
}

}  // namespace fdp
