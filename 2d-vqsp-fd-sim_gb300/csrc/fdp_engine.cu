// C ABI of the GB300 time-stepping engine (declared in include/fdp.h).
//
// A context holds one shot's grid resident in HBM: the eight wavefield
// arrays, the medium, the PML profiles and memory variables, the bottom
// history, the source time function and the receiver samples.  fdp_run
// enqueues each time level's kernels on the context's stream (with the
// frame/core split: each phase's frame kernel on a side stream beside its
// core kernel, the row-1/receiver step folded into the next level's stress
// frame kernel, one k_edge at the end of a run); runs of kChunk levels are
// captured once into a CUDA graph and replayed.  Batches (fdp_batch_*)
// advance many contexts together: work-queue kernels over all shots, or
// every shot's own level sequence side by side in one graph.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <type_traits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "fdp.h"
#include "fdp_ctx.h"
#include "fdp_core_tma.cuh"
#include "fdp_march.cuh"

using fdp::Params;
using fdp::kPadX;
using fdp::kPadZ;

namespace {

constexpr int kChunk = 32;       // time levels per captured graph
constexpr int kBlockX = 128;     // threads per block (x)

// Message of the last failed call that has no context, per host thread, so
// concurrent callers neither race on it nor see each other's messages.
thread_local std::string g_create_error;

}  // namespace

namespace fdp {
// Error message of calls that have no context (fdp_create, fdp_receivers_noalloc).
void set_global_error(const char* msg) { g_create_error = msg; }
}  // namespace fdp

namespace {

int fail(fdp_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (c) c->err = buf; else g_create_error = buf;
  return code;
}

#define CK(c, call)                                                                         \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) return fail((c), FDP_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

int dev_alloc(fdp_ctx* c, DevArr& a, size_t bytes) {
  if (a.p) { cudaFree(a.p); a.p = nullptr; a.bytes = 0; }
  if (bytes == 0) return FDP_OK;
  cudaError_t e = cudaMalloc(&a.p, bytes);
  if (e != cudaSuccess) return fail(c, FDP_ERR_ALLOC, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
  a.bytes = bytes;
  e = cudaMemsetAsync(a.p, 0, bytes, c->stream);
  if (e != cudaSuccess) return fail(c, FDP_ERR_CUDA, "cudaMemsetAsync: %s", cudaGetErrorString(e));
  return FDP_OK;
}

// Bounds (lx, ux, lz, uz) of every field id, as the reference allocates them.
bool bounds_of(const fdp_ctx* c, int id, int b[4]) {
  const int PMLL = c->PMLL, PMLXH = c->PMLXH, PMLZH = c->PMLZH, MX = c->MX, TPML = c->TPML;
  auto set = [&](int a, int bb, int cc, int d) { b[0] = a; b[1] = bb; b[2] = cc; b[3] = d; return true; };
  switch (id) {
    case FDP_UM: case FDP_WM: case FDP_QX: case FDP_QZ:
    case FDP_TXX: case FDP_TZZ: case FDP_TXZ: case FDP_PRES:
    case FDP_QXP: case FDP_QZP:
      return set(PMLL, PMLXH, 0, PMLZH);
    case FDP_PZXL: return set(PMLL, 2, 0, PMLZH);
    case FDP_PZXH: return set(MX, PMLXH, 0, PMLZH);
    case FDP_PXXL: case FDP_OXXL: return set(PMLL, 1, 0, PMLZH);
    case FDP_PXXH: case FDP_OXXH: return set(MX, PMLXH, 0, PMLZH);
    case FDP_PXZH: return set(PMLL, PMLXH, 0, TPML + 1);
    case FDP_PZZH: case FDP_OZZH: return set(PMLL, PMLXH, 0, TPML);
    case FDP_RXXL: case FDP_SXXL: case FDP_GXXL: case FDP_HXXL: return set(PMLL, 3, 0, PMLZH);
    case FDP_RXXH: case FDP_SXXH: case FDP_GXXH: case FDP_HXXH: return set(MX - 1, PMLXH, 0, PMLZH);
    case FDP_RZXL: case FDP_GZXL: return set(PMLL, 2, 0, PMLZH);
    case FDP_RZXH: case FDP_GZXH: return set(MX - 1, PMLXH, 0, PMLZH);
    case FDP_RXZH: case FDP_GXZH: case FDP_RZZH: case FDP_SZZH: case FDP_GZZH: case FDP_HZZH:
      return set(PMLL, PMLXH, 0, TPML);
    case FDP_SZ_U: case FDP_SZ_W: case FDP_SZ_QX: case FDP_SZ_QZ:
      return set(PMLL, PMLXH, 0, 2);
    default: return false;
  }
}

// All copies go through the context's stream (which does not synchronise
// with the legacy default stream) and wait for completion.
int copy_sync(fdp_ctx* c, void* dst, const void* src, size_t bytes, cudaMemcpyKind kind) {
  if (bytes == 0) return FDP_OK;
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, kind, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(c, FDP_ERR_CUDA, "copy of %zu bytes: %s", bytes, cudaGetErrorString(e));
  return FDP_OK;
}

int copy2d_sync(fdp_ctx* c, void* dst, size_t dpitch, const void* src, size_t spitch, size_t w, size_t h,
                cudaMemcpyKind kind) {
  cudaError_t e = cudaMemcpy2DAsync(dst, dpitch, src, spitch, w, h, kind, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(c, FDP_ERR_CUDA, "2-D copy: %s", cudaGetErrorString(e));
  return FDP_OK;
}

size_t count_of(const int b[4]) { return (size_t)(b[1] - b[0] + 1) * (size_t)(b[3] - b[2] + 1); }

// TMA descriptor of one padded field (whole allocation, boxes of bw x bh
// elements).  cuTensorMapEncodeTiled is reached through the runtime's
// driver entry point, so the library does not link libcuda itself.
int make_field_map(fdp_ctx* c, CUtensorMap* map, void* base, int bw = fdp::kSX, int bh = fdp::kSZ) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn)
      return fail(c, FDP_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  const cuuint64_t dims[2] = {(cuuint64_t)c->pitch, (cuuint64_t)c->rows_alloc};
  const cuuint64_t strides[1] = {(cuuint64_t)c->pitch * (cuuint64_t)c->prec};
  const cuuint32_t box[2] = {(cuuint32_t)bw, (cuuint32_t)bh};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode(map, c->prec == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2,
                            base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(c, FDP_ERR_CUDA, "cuTensorMapEncodeTiled failed (CUresult %d)", (int)r);
  return FDP_OK;
}

// Maps of the TMA-staged core kernels (fdp_core_tma.cuh), built once the
// medium is known: FP32 fields and the 10 Biot planes.  Phase 0 reads u, w,
// qx, qz and updates the stresses; phase 1 reads the stresses and updates
// qx, u, qz, w.
int make_core_maps(fdp_ctx* c) {
  c->core_tma = false;
  if (!c->core_tma_req || c->prec != 4 || c->medium_mode != fdp::M_BIOT) return FDP_OK;
  static const int in[2][4] = {{0, 1, 2, 3}, {4, 5, 6, 7}};
  static const int upd[2][4] = {{4, 5, 6, 7}, {2, 0, 3, 1}};
  const size_t pstride = (size_t)c->rows_alloc * c->pitch;
  int rc;
  for (int ph = 0; ph < 2; ++ph) {
    fdp::CoreMaps& m = c->cmaps[ph];
    for (int k = 0; k < 4; ++k) {
      if ((rc = make_field_map(c, &m.m[k], c->fields[in[ph][k]].p, fdp::kCHW, fdp::core_box_rows(ph, k))) != FDP_OK)
        return rc;
      if ((rc = make_field_map(c, &m.m[4 + k], c->fields[upd[ph][k]].p, fdp::kCTW, fdp::kCTH)) != FDP_OK) return rc;
    }
    for (int k = 0; k < 5; ++k)
      if ((rc = make_field_map(c, &m.m[8 + k], (float*)c->planes.p + (size_t)(5 * ph + k) * pstride, fdp::kCTW,
                               fdp::kCTH)) != FDP_OK)
        return rc;
  }
  int dev = 0, nsm = 0;
  CK(c, cudaGetDevice(&dev));
  CK(c, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  CK(c, cudaFuncSetAttribute(fdp::k_core_tma<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fdp::kCoreTmaSmem));
  CK(c, cudaFuncSetAttribute(fdp::k_core_tma<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fdp::kCoreTmaSmem));
  c->core_ctas = nsm;
  c->core_tma = true;
  return FDP_OK;
}

// Waits for the context's work and reports a kernel whose bounded wait
// expired (the status word the kernels set instead of hanging).
int device_status(fdp_ctx* c) {
  CK(c, cudaStreamSynchronize(c->stream));
  int v = 0;
  CK(c, cudaMemcpyAsync(&v, c->errbuf.p, sizeof v, cudaMemcpyDeviceToHost, c->stream));
  CK(c, cudaStreamSynchronize(c->stream));
  if (v) {
    // reported once: the word is cleared, and the context stays usable
    CK(c, cudaMemsetAsync(c->errbuf.p, 0, sizeof v, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return fail(c, FDP_ERR_DEVICE, "a kernel gave up waiting (status %d)", v);
  }
  return FDP_OK;
}

template <class T> void fill_params(fdp_ctx* c, Params<T>& p) {
  std::memset(&p, 0, sizeof p);
  p.MX = c->MX; p.MZ = c->MZ; p.TPML = c->TPML; p.PMLL = c->PMLL; p.PMLXH = c->PMLXH; p.PMLZH = c->PMLZH;
  p.NX = c->NX; p.NZ = c->NZ; p.MX1 = c->MX1; p.LIN_X = c->g.lin_x; p.LIN_Z = c->g.lin_z;
  p.pitch = c->pitch;
  p.cs_x0 = c->cs[0]; p.cs_x1 = c->cs[1]; p.cs_z0 = c->cs[2]; p.cs_z1 = c->cs[3];
  p.cv_x0 = c->cv[0]; p.cv_x1 = c->cv[1]; p.cv_z0 = c->cv[2]; p.cv_z1 = c->cv[3];
  // mod_auxil.F90:19-20 (default-real constants) and aux1.F90:44-46
  const T H = (T)c->g.h;
  p.A = (T)(-1.0f / 24.0f);
  p.B = (T)(9.0f / 8.0f);
  p.AH = p.A / H; p.BH = p.B / H; p.CH = T(1) / H;
  p.BC = p.BH / p.CH;  // strain_uw_zz.F90:45
  p.DT = (T)c->g.dt;
  p.DTE = p.DT + (T)c->g.tau_eps;
  const size_t off = (size_t)kPadZ * c->pitch + kPadX;
  T** f[8] = {&p.UM, &p.WM, &p.QX, &p.QZ, &p.TXX, &p.TZZ, &p.TXZ, &p.PRES};
  T** o[8] = {&p.oUM, &p.oWM, &p.oQX, &p.oQZ, &p.oTXX, &p.oTZZ, &p.oTXZ, &p.oPRES};
  for (int k = 0; k < 8; ++k) *f[k] = *o[k] = (T*)c->fields[k].p + off;
  p.JM = c->jm.p ? (const int32_t*)c->jm.p + off : nullptr;
  p.coef = (const T*)c->coef.p;
  p.cld = c->jmnum + 1;
  p.planes = c->planes.p ? (const T*)c->planes.p + off : nullptr;
  p.pstride = (long long)c->rows_alloc * c->pitch;
  for (int k = 0; k < fdp::C_NCOEF; ++k) {
    p.src[k] = c->src[k];
    p.neg[k] = c->neg[k];
    p.cval[k] = sizeof(T) == 8 ? (T)c->cval_d[k] : (T)c->cval_f[k];
  }
  p.AUX = (const T*)c->aux.p;
  for (int k = 0; k < fdp::C_NCOEF; ++k)
    p.cptr[k] = (p.planes && c->src[k] >= 0) ? p.planes + (long long)c->src[k] * p.pstride : nullptr;
  for (int s = 0; s < 10; ++s)
    p.bplane[s] = (c->medium_mode == fdp::M_BIOT) ? p.planes + (long long)s * p.pstride : nullptr;
  const T** pr[24] = {&p.ODA_XL, &p.ODB_XL, &p.ODC_XL, &p.ODD_XL, &p.ODA_XH, &p.ODB_XH, &p.ODC_XH, &p.ODD_XH,
                      &p.ODA_ZH, &p.ODB_ZH, &p.ODC_ZH, &p.ODD_ZH,
                      &p.ODA2_XL, &p.ODB2_XL, &p.ODC2_XL, &p.ODD2_XL, &p.ODA2_XH, &p.ODB2_XH, &p.ODC2_XH, &p.ODD2_XH,
                      &p.ODA2_ZH, &p.ODB2_ZH, &p.ODC2_ZH, &p.ODD2_ZH};
  for (int k = 0; k < 24; ++k) *pr[k] = (const T*)c->prof[k].p;
  T** m[27] = {&p.PZXL, &p.PZXH, &p.PXXL, &p.PXXH, &p.OXXL, &p.OXXH, &p.PXZH, &p.PZZH, &p.OZZH,
               &p.RXXL, &p.RXXH, &p.SXXL, &p.SXXH, &p.RZXL, &p.RZXH, &p.GXXL, &p.GXXH, &p.HXXL, &p.HXXH,
               &p.GZXL, &p.GZXH, &p.RXZH, &p.GXZH, &p.RZZH, &p.SZZH, &p.GZZH, &p.HZZH};
  for (int k = 0; k < 27; ++k) *m[k] = (T*)c->mem[k].p;
  p.AB = (const T*)c->ab.p;
  p.HIST = (T*)c->hist.p;
  p.STF = (const T*)c->stf.p;
  p.MT2 = c->mt2;
  p.it_base = (const int*)c->itbase.p;
  p.MR = c->mr;
  p.REC = (const int*)c->rec.p;
  p.RAW = (T*)c->raw.p;
  p.err = (int*)c->errbuf.p;
}

dim3 cell_grid(const fdp_ctx* c, int kind) {
  const int rows = fdp::kBZ * (kind == 0 ? fdp::kRZS : fdp::kRZV);  // rows per block
  return dim3((c->NX + fdp::kBX - 1) / fdp::kBX, (c->NZ + rows - 1) / rows, 1);
}

int edge_threads(const fdp_ctx* c) { return (c->g.stress_imaging ? c->NX : 0) + c->mr; }

// kind 0 = stress phase, 1 = velocity phase, 2 = edge (imaging row 1 and receivers)
dim3 tile_grid(const fdp_ctx* c) {
  return dim3((c->NX + fdp::kTX - 1) / fdp::kTX, (c->NZ + fdp::kTZ - 1) / fdp::kTZ, 1);
}

// core grid of a phase: 4 cells per thread along x
dim3 core_grid(const int r[4]) {
  const int threads_x = (r[1] - r[0]) / 4;
  return dim3((threads_x + fdp::kBX - 1) / fdp::kBX, (r[3] - r[2] + fdp::kBZ - 1) / fdp::kBZ, 1);
}

// The TMA-staged core kernel of phase `kind`, where the context uses it
// (FP32, Biot planes); false leaves the phase to the per-thread-load core.
template <class T, int MODE> bool launch_core_tma(fdp_ctx* c, const Params<T>& p, int kind) {
  if constexpr (std::is_same<T, float>::value && MODE == fdp::M_BIOT) {
    if (!c->core_tma) return false;
    const dim3 blk(fdp::kBX, fdp::kBZ, 1);
    const int g = std::min(fdp::core_tiles(p, kind).n, c->core_ctas);
    if (kind == 0) fdp::k_core_tma<0><<<g, blk, fdp::kCoreTmaSmem, c->stream>>>(p, c->cmaps[0]);
    else fdp::k_core_tma<1><<<g, blk, fdp::kCoreTmaSmem, c->stream>>>(p, c->cmaps[1]);
    return true;
  }
  return false;
}

// Launch modes of the frame/core split (launch_level_any): the stress frame
// kernel finishes the previous level (row 1, velocity samples), and the
// velocity frame kernel takes this level's stress samples (k_edge then
// skips them).
constexpr int kDeferPrev = 1, kFrameSamples = 2;

template <class T, bool SI, int MODE> void launch_kind(fdp_ctx* c, const Params<T>& p, int kind, int it_off, int mode) {
  const dim3 blk(fdp::kBX, fdp::kBZ, 1);
  const dim3 tblk(fdp::kTX, 4, 1);
  if (kind == 0 && c->use_tma) fdp::k_stress_tma<T, SI, MODE><<<tile_grid(c), tblk, 0, c->stream>>>(p, c->tma_vel, it_off);
  else if (kind == 1 && c->use_tma) fdp::k_velocity_tma<T, SI, MODE><<<tile_grid(c), tblk, 0, c->stream>>>(p, c->tma_str, it_off);
  else if ((kind == 0 || kind == 1) && c->use_core && c->fused[kind]) {
    const int* r = kind == 0 ? c->cs : c->cv;
    fdp::FusedGrid g{};
    g.units = (const int4*)(kind == 0 ? c->frame_s.p : c->frame_v.p);
    g.nframe = kind == 0 ? c->nframe_s : c->nframe_v;
    const dim3 cg = r[1] > r[0] ? core_grid(r) : dim3(0, 0, 1);
    g.gx = (int)cg.x;
    g.ncore = (int)(cg.x * cg.y);
    g.per = g.nframe > 0 ? (g.ncore + g.nframe - 1) / g.nframe : 0;
    const int total = g.nframe > 0 ? g.nframe * (g.per + 1) : g.ncore;
    if (kind == 0) fdp::k_stress_fused<T, SI, MODE><<<total, blk, 0, c->stream>>>(p, g, it_off);
    else fdp::k_velocity_fused<T, SI, MODE><<<total, blk, 0, c->stream>>>(p, g);
  }
  else if ((kind == 0 || kind == 1) && c->use_core) {
    const int* r = kind == 0 ? c->cs : c->cv;
    const bool core = r[1] > r[0];
    cudaStream_t fs = core ? c->side : c->stream;
    if (core) {
      cudaEventRecord(c->fork, c->stream);
      cudaStreamWaitEvent(c->side, c->fork, 0);
    }
    const int mr_blocks = (c->mr + fdp::kBX * fdp::kBZ - 1) / (fdp::kBX * fdp::kBZ);
    if (kind == 0)
      fdp::k_stress_frame<T, SI, MODE><<<c->nframe_s + ((mode & kDeferPrev) ? mr_blocks : 0), blk, 0, fs>>>(
          p, (const int4*)c->frame_s.p, c->nframe_s, it_off, (mode & kDeferPrev) ? 1 : 0);
    else
      fdp::k_velocity_frame<T, SI, MODE><<<c->nframe_v + ((mode & kFrameSamples) ? mr_blocks : 0), blk, 0, fs>>>(
          p, (const int4*)c->frame_v.p, c->nframe_v, it_off);
    if (core) {
      if (c->core_ev[kind][0]) cudaEventRecord(c->core_ev[kind][0], c->stream);
      if (launch_core_tma<T, MODE>(c, p, kind)) {}
      else if (kind == 0) fdp::k_stress_core<T, MODE><<<core_grid(r), blk, 0, c->stream>>>(p);
      else fdp::k_velocity_core<T, MODE><<<core_grid(r), blk, 0, c->stream>>>(p);
      if (c->core_ev[kind][1]) cudaEventRecord(c->core_ev[kind][1], c->stream);
      cudaEventRecord(c->join, c->side);
      cudaStreamWaitEvent(c->stream, c->join, 0);
      c->launches += 1;
    }
  }
  else if (kind == 0) fdp::k_stress<T, SI, MODE><<<cell_grid(c, 0), blk, 0, c->stream>>>(p, it_off);
  else if (kind == 1) fdp::k_velocity<T, SI, MODE><<<cell_grid(c, 1), blk, 0, c->stream>>>(p, it_off);
  else fdp::k_edge<T, SI><<<(edge_threads(c) + kBlockX - 1) / kBlockX, kBlockX, 0, c->stream>>>(
      p, it_off, (mode & kFrameSamples) ? 0 : 1);
  c->launches += 1;
}

// Frame unit lists of the frame kernels beside core rectangles cs (stress)
// and cv (velocity): the columns split at the cores' edges ([PMLL, x0),
// [x0, x1), [x1, PMLXH]) so that no unit straddles a core edge, units of
// kBX columns from each segment's start; a unit is listed when it holds a
// cell outside the core (or, when the stress core leaves the source row to
// the frame, a cell of the source row).
int build_units(fdp_ctx* c, const int cs[4], const int cv[4], bool src_in_core, DevArr& frame_s, int& nframe_s,
                DevArr& frame_v, int& nframe_v) {
  auto in = [](const int r[4], int I, int L) { return I >= r[0] && I < r[1] && L >= r[2] && L < r[3]; };
  std::vector<int> us, uv;
  for (int ph = 0; ph < 2; ++ph) {
    const int rows = fdp::kBZ * (ph == 0 ? fdp::kRZS : fdp::kRZV);
    const int gy = (c->NZ + rows - 1) / rows;
    const int* r = ph == 0 ? cs : cv;
    std::vector<int>& out = ph == 0 ? us : uv;
    std::vector<std::pair<int, int>> segs;
    if (r[1] > r[0]) segs = {{c->PMLL, r[0]}, {r[0], r[1]}, {r[1], c->PMLXH + 1}};
    else segs = {{c->PMLL, c->PMLXH + 1}};
    // stress: units of kBZ*kRZS rows from row 0 down; velocity: units of
    // kBZ rows with one row per thread up to row PMLZH-3 (short threads for
    // the latency-bound PML cells), then the bottom three rows, one column
    // per thread, kBX*kBZ columns per unit
    if (ph == 1)
      for (int I0 = c->PMLL; I0 <= c->PMLXH; I0 += fdp::kBX * fdp::kBZ) {
        out.push_back(I0); out.push_back(std::min(I0 + fdp::kBX * fdp::kBZ, c->PMLXH + 1));
        out.push_back(0); out.push_back(2);
      }
    const int nbands = ph == 0 ? gy : (c->PMLZH - 3 + 1 + fdp::kBZ - 1) / fdp::kBZ;
    for (int by = 0; by < nbands; ++by) {
      int la, lb, tag, w;
      if (ph == 0) { la = by * rows; lb = la + rows - 1; tag = by; w = 0; }
      else { la = by * fdp::kBZ; lb = std::min(la + fdp::kBZ - 1, c->PMLZH - 3); tag = la; w = 1; }
      for (const auto& sg : segs)
        for (int I0 = sg.first; I0 < sg.second; I0 += fdp::kBX) {
          const int I1 = std::min(I0 + fdp::kBX, sg.second);
          const int lo = std::max(la, 0), hi = std::min(lb, c->PMLZH);
          bool frame = false;
          if (lo <= hi)
            frame = !(in(r, I0, lo) && in(r, I1 - 1, hi)) ||
                    (ph == 0 && !src_in_core && c->g.lin_z >= lo && c->g.lin_z <= hi);
          if (frame) { out.push_back(I0); out.push_back(I1); out.push_back(tag); out.push_back(w); }
        }
    }
  }
  nframe_s = (int)us.size() / 4;
  nframe_v = (int)uv.size() / 4;
  int rc;
  if ((rc = dev_alloc(c, frame_s, us.size() * sizeof(int))) != FDP_OK) return rc;
  if ((rc = dev_alloc(c, frame_v, uv.size() * sizeof(int))) != FDP_OK) return rc;
  if ((rc = copy_sync(c, frame_s.p, us.data(), us.size() * sizeof(int), cudaMemcpyHostToDevice)) != FDP_OK) return rc;
  return copy_sync(c, frame_v.p, uv.data(), uv.size() * sizeof(int), cudaMemcpyHostToDevice);
}

// The march variant's region F and its launch (see fdp_march.cuh); false
// when the context cannot run it (FP64, a grid too small for a region F).
bool plan_march(fdp_ctx* c) {
  if (c->prec != 4) return false;
  // The new stresses the march kernel computes two cells and two rows
  // around F are interior ones (columns 3..MX-2 and rows from 2,
  // strain_uw_xx.F90:80, time_loop.F90:93-124), as are the velocities of F
  // (columns 4..MX-2, inh_qx_int.F90:40).  Its first halo row of stresses
  // (two above F) reads velocities from four rows above F on, which stays
  // below the stress-imaging row 1 that the stress frame kernel writes
  // meanwhile.  The frame kernels write the new stresses of a band of one
  // vector and two rows along F's edges, and every cell outside F.
  int fx0 = 5;
  while ((fx0 - c->PMLL) % 4 != 0) ++fx0;
  const int nvec = (c->MX - 3 - fx0) / 4;
  const int fz0 = 6, fz1 = c->MZ - 3;
  if (nvec < 3 || fz1 - fz0 < 5) return false;
  const int fx1 = fx0 + 4 * nvec;
  fdp::MarchGrid& m = c->mg;
  m.fx0 = fx0; m.fx1 = fx1; m.fz0 = fz0; m.fz1 = fz1;
  m.sx0 = fx0 + 4; m.sx1 = fx1 - 4; m.sz0 = fz0 + 2; m.sz1 = fz1 - 2;
  m.nvec = nvec;
  m.nstrips = (nvec + fdp::kMarchVec - 1) / fdp::kMarchVec;
  m.total = (long long)m.nstrips * (fz1 - fz0);
  c->ms[0] = m.sx0; c->ms[1] = m.sx1; c->ms[2] = m.sz0; c->ms[3] = m.sz1;
  c->mv[0] = fx0; c->mv[1] = fx1; c->mv[2] = fz0; c->mv[3] = fz1;
  return true;
}

// The march launch for the context's medium, once it is set: whether its
// levels run as march levels, the band height and the CTAs.
template <int MODE> bool march_shape_for(fdp_ctx* c) {
  fdp::MarchGrid& m = c->mg;
  int sms = 152, l2 = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->g.device);
  if (const char* es = std::getenv("FDP_MARCH_SMS")) sms = std::max(1, std::min(sms, std::atoi(es)));  // plan for fewer SMs
  cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c->g.device);
  // Unless named, march levels run only where a level's data outgrow L2:
  // below that the split's second phase finds the first phase's output in
  // L2.  Measured on layered grids with Biot planes (104 B per cell of F):
  // 1280^2 (166 MB per level in the march kernel, L2 129 MB) split 0.0379
  // ms, march 0.0410; 1408^2 (204 MB) 0.0476 and 0.0472; 2048^2 0.0967 and
  // 0.0833.  Other media: the 16 field values and a material index (table)
  // or the distinct coefficient planes (planes mode) per cell.
  const double per_cell = 64.0 + (MODE == fdp::M_BIOT ? 40.0 : MODE == fdp::M_TABLE ? 4.0 : 4.0 * c->nplanes);
  const double level_bytes = (double)m.nvec * 4 * (m.fz1 - m.fz0) * per_cell;
  if (!c->march_forced && level_bytes < 1.5 * l2) return false;
  // the same number of CTAs on every strip, each a contiguous range of the
  // strip's rows (or, with more strips than CTA slots, the same number of
  // whole strips per CTA): the CTAs then march down the same rows of every
  // strip together, and the boxes they read at a time make up whole rows of
  // the arrays.  Measured with bands of 8 rows: 2816^2 (24 strips) at 152
  // CTAs, whose ranges drift against the strips, 0.196 ms per level; at 144
  // (six per strip) 0.145 ms.  aligned(slots) = the CTAs and the range of
  // each (0: the strips' rows split evenly), and the share of the slots'
  // time they fill.
  const int H = m.fz1 - m.fz0;
  struct Split { long long ctas, span; double fill; };
  auto aligned = [&](long long slots) -> Split {
    if (m.nstrips <= slots) {
      const long long n = slots / m.nstrips * m.nstrips;
      return {n, 0, (double)n / slots};
    }
    const long long q = (m.nstrips + slots - 1) / slots;  // strips per CTA
    return {(m.nstrips + q - 1) / q, q * H, (double)m.nstrips / ((double)q * slots)};
  };
  using S4 = fdp::MarchShapeOf<MODE, 4>;
  using S6 = fdp::MarchShapeOf<MODE, 6>;
  using S8 = fdp::MarchShapeOf<MODE, 8>;
  // bands of 8 rows (one CTA of eight warps per SM) or of 4 (two CTAs of
  // four warps per SM with the Biot planes staged, three without),
  // whichever keeps more warps busy: warps per SM times the share of the
  // slots the strips fill (8 on a near tie); 6 (six warps) on request.
  // Biot planes: 2048^2 (17 strips) 136 CTAs of 8 rows 0.0853 ms per level,
  // 289 of 4 rows 0.0833; 4096^2 (34 strips) 136 CTAs of 8 rows 0.2900 ms,
  // 272 of 4 rows 0.2955.
  const char* er = std::getenv("FDP_MARCH_ROWS");
  const int rows = er ? std::atoi(er) : 0;
  if (rows == 4 || rows == 6 || rows == 8) c->march_rows = rows;
  else {
    const double w4 = 4.0 * S4::kCtasPerSm * aligned((long long)sms * S4::kCtasPerSm).fill;
    const double w8 = 8.0 * S8::kCtasPerSm * aligned((long long)sms * S8::kCtasPerSm).fill;
    c->march_rows = w4 > 1.02 * w8 ? 4 : 8;
  }
  int per_sm = 1;
  cudaError_t e = cudaSuccess;
  auto shape = [&](auto kernel, size_t smem, int ctas_per_sm) {
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    per_sm = ctas_per_sm;
  };
  if (c->march_rows == 4) shape(fdp::k_march<MODE, 4>, S4::kSmem, S4::kCtasPerSm);
  else if (c->march_rows == 6) shape(fdp::k_march<MODE, 6>, S6::kSmem, S6::kCtasPerSm);
  else shape(fdp::k_march<MODE, 8>, S8::kSmem, S8::kCtasPerSm);
  if (e != cudaSuccess) return false;
  const Split sp = aligned((long long)sms * per_sm);
  const char* ec = std::getenv("FDP_MARCH_CTAS");
  m.span = ec ? 0 : sp.span;
  c->march_ctas = (int)std::min<long long>(ec ? std::max(1, std::atoi(ec)) : sp.ctas, m.total);
  return true;
}

bool march_shape(fdp_ctx* c) {
  switch (c->medium_mode) {
    case fdp::M_BIOT: return march_shape_for<fdp::M_BIOT>(c);
    case fdp::M_TABLE: return march_shape_for<fdp::M_TABLE>(c);
    default: return march_shape_for<fdp::M_PLANES>(c);
  }
}

// The second buffer of each wavefield array, made as a copy of the first
// when the context first gets a medium its march levels run with: cells no
// level updates are then read from either.  false (nothing held, no error
// recorded) when the device has no room; the context keeps the split.
bool alloc_alt(fdp_ctx* c) {
  if (c->alt[0].p) return true;
  for (int k = 0; k < 8; ++k) {
    const size_t bytes = c->fields[k].bytes;
    cudaError_t e = cudaMalloc(&c->alt[k].p, bytes);
    if (e == cudaSuccess) {
      c->alt[k].bytes = bytes;
      e = cudaMemcpyAsync(c->alt[k].p, c->fields[k].p, bytes, cudaMemcpyDeviceToDevice, c->stream);
    }
    if (e != cudaSuccess) {
      cudaGetLastError();
      for (auto& a : c->alt)
        if (a.p) { cudaFree(a.p); a.p = nullptr; a.bytes = 0; }
      return false;
    }
  }
  return true;
}

// The march launch and the march kernel's tensor maps for each of the two
// buffers of the fields (indexed like cur) and, for a medium held as Biot
// planes, of the planes; the march levels run once the medium is set and
// its launch chosen (a grid whose levels stay in L2, or a device without
// room for the second buffers, leaves the context on the frame/core split).
int make_march_maps(fdp_ctx* c) {
  c->march_ready = false;
  if (!c->march) return FDP_OK;
  const bool biot = c->medium_mode == fdp::M_BIOT;
  if (biot && !c->planes.p) return FDP_OK;
  if (!march_shape(c)) return FDP_OK;
  if (!alloc_alt(c)) return FDP_OK;
  const size_t pstride = (size_t)c->rows_alloc * c->pitch;
  int rc;
  for (int b = 0; b < 2; ++b) {
    const DevArr* f = b == c->cur ? c->fields : c->alt;
    fdp::MarchMaps& m = c->mmaps[b];
    for (int k = 0; k < 8; ++k)
      if ((rc = make_field_map(c, &m.f[k], f[k].p, fdp::kMarchW, c->march_rows)) != FDP_OK) return rc;
    for (int k = 0; k < 10 && biot; ++k)
      if ((rc = make_field_map(c, &m.pl[k], (float*)c->planes.p + (size_t)k * pstride, fdp::kMarchW,
                               c->march_rows)) != FDP_OK)
        return rc;
  }
  c->march_ready = true;
  return FDP_OK;
}

// Core rectangles and frame unit lists.  A core cell of the stress phase
// needs 3 <= I <= MX-2, 2 <= L <= MZ-2, L != LIN_Z; of the velocity phase
// 4 <= I <= MX-2, 2 <= L <= MZ-2 (the interior branches).  The core starts
// on a 16-byte-aligned column and spans whole groups of four.  With the
// march variant, also F and the frame units beside it.
int plan_core(fdp_ctx* c) {
  auto rect = [&](int r[4], int xmin, int zmin) {
    int x0 = xmin;
    while ((x0 - c->PMLL) % 4 != 0) ++x0;
    const int n4 = (c->MX - 2 - x0 + 1) / 4;
    r[0] = x0; r[1] = x0 + 4 * std::max(n4, 0);
    r[2] = zmin; r[3] = c->MZ - 1;
    if (r[1] <= r[0] || r[3] <= r[2]) { r[0] = r[1] = r[2] = r[3] = 0; }
  };
  // under stress imaging, rows 2..4 stay with the stress frame, whose unit
  // holding them also writes the mirror rows 0 and 1 from them
  rect(c->cs, 3, c->g.stress_imaging ? 5 : 2);
  rect(c->cv, 4, 2);
  int rc = build_units(c, c->cs, c->cv, false, c->frame_s, c->nframe_s, c->frame_v, c->nframe_v);
  if (rc != FDP_OK) return rc;
  if (c->march && !plan_march(c)) c->march = false;  // the frame/core split runs the context
  if (c->march) rc = build_units(c, c->ms, c->mv, true, c->mframe_s, c->nmframe_s, c->mframe_v, c->nmframe_v);
  return rc;
}

template <class T> void launch(fdp_ctx* c, const Params<T>& p, int kind, int it_off, int mode = 0) {
  const bool si = c->g.stress_imaging != 0;
  switch (c->medium_mode) {
    case fdp::M_TABLE:
      si ? launch_kind<T, true, fdp::M_TABLE>(c, p, kind, it_off, mode)
         : launch_kind<T, false, fdp::M_TABLE>(c, p, kind, it_off, mode);
      break;
    case fdp::M_BIOT:
      si ? launch_kind<T, true, fdp::M_BIOT>(c, p, kind, it_off, mode)
         : launch_kind<T, false, fdp::M_BIOT>(c, p, kind, it_off, mode);
      break;
    default:
      si ? launch_kind<T, true, fdp::M_PLANES>(c, p, kind, it_off, mode)
         : launch_kind<T, false, fdp::M_PLANES>(c, p, kind, it_off, mode);
  }
}

// Whether the levels run as march levels: the march variant planned a deep
// interior and has its tensor maps, and neither a batch (whose work-queue
// kernels update in place; its shots mode runs march levels in pairs) nor
// an attached learned edge (whose kernels work on the current buffers after
// every level) holds the context.
bool use_march(const fdp_ctx* c) {
  return c->march && c->march_ready && (!c->in_batch || c->batch_march) && !(c->edge && c->edge_attached);
}

// After a march level the other buffers are current.
void flip_buffers(fdp_ctx* c) {
  for (int k = 0; k < 8; ++k) std::swap(c->fields[k], c->alt[k]);
  c->cur ^= 1;
}

// Whether a run of levels folds the row-1/receiver step of each level into
// the next level's stress frame kernel (and its stress samples into the
// level's velocity frame kernel), leaving one k_edge at the end of the run:
// the frame/core split with no learned edge attached (that one reads row 1
// after every level).
bool defer_edge(const fdp_ctx* c) {
  return c->use_core && !c->use_tma && !c->fused[0] && !c->fused[1] && !(c->edge && c->edge_attached) &&
         edge_threads(c) > 0;
}

// The wavefield pointers of p: reads from `in`, the phase's new values to
// `out` (arrays of the eight fields UM WM QX QZ TXX TZZ TXZ PRES).
template <class T> void set_fields(const fdp_ctx* c, Params<T>& p, const DevArr* in, const DevArr* out) {
  const size_t off = (size_t)kPadZ * c->pitch + kPadX;
  T** f[8] = {&p.UM, &p.WM, &p.QX, &p.QZ, &p.TXX, &p.TZZ, &p.TXZ, &p.PRES};
  T** o[8] = {&p.oUM, &p.oWM, &p.oQX, &p.oQZ, &p.oTXX, &p.oTZZ, &p.oTXZ, &p.oPRES};
  for (int k = 0; k < 8; ++k) {
    *f[k] = (T*)in[k].p + off;
    *o[k] = (T*)out[k].p + off;
  }
}

// One level of the march variant: the stress and then the velocity frame
// kernel on the side stream, beside the march kernel over the deep interior
// on the context's stream; every kernel reads the current buffers (A) and
// writes the other ones (B), which are current after the level.  The
// stress frame kernel also finishes the previous level of the run (row 1,
// the velocity and the stress samples of the receivers: both stay in A
// through this level); the run's last level is finished by k_edge.
template <class T, bool SI, int MODE>
void launch_level_march(fdp_ctx* c, const Params<T>& base, int it_off, bool first, bool last) {
  const DevArr* A = c->fields;
  const DevArr* B = c->alt;
  DevArr sv[8];  // velocities in A, stresses in B
  for (int k = 0; k < 8; ++k) sv[k] = k < 4 ? A[k] : B[k];
  Params<T> ps = base;
  ps.cs_x0 = c->ms[0]; ps.cs_x1 = c->ms[1]; ps.cs_z0 = c->ms[2]; ps.cs_z1 = c->ms[3];
  ps.cv_x0 = c->mv[0]; ps.cv_x1 = c->mv[1]; ps.cv_z0 = c->mv[2]; ps.cv_z1 = c->mv[3];
  ps.cs_src = 1;  // the march kernel adds the source term itself
  Params<T> pv = ps, pm = ps;
  set_fields(c, ps, A, sv);   // stresses A -> B; velocities read (row 1 finished) in A
  set_fields(c, pv, sv, B);   // reads the new stresses (B) and the old velocities (A)
  set_fields(c, pm, A, B);
  const dim3 blk(fdp::kBX, fdp::kBZ, 1);
  const bool defer = !first && edge_threads(c) > 0;
  const int mr_blocks = (c->mr + fdp::kBX * fdp::kBZ - 1) / (fdp::kBX * fdp::kBZ);
  // the march kernel is enqueued first, so that its CTAs, which march in
  // step with one another, take their SM slots before the frame kernels'
  // blocks fill the rest (layered 2048^2: 0.0787 ms per level; frame
  // kernels first 0.0840 ms)
  cudaEventRecord(c->fork, c->stream);
  cudaStreamWaitEvent(c->side, c->fork, 0);
  if (c->core_ev[0][0]) cudaEventRecord(c->core_ev[0][0], c->stream);
  if constexpr (std::is_same<T, float>::value) {
    using S4 = fdp::MarchShapeOf<MODE, 4>;
    using S6 = fdp::MarchShapeOf<MODE, 6>;
    using S8 = fdp::MarchShapeOf<MODE, 8>;
    if (c->march_rows == 8)
      fdp::k_march<MODE, 8><<<c->march_ctas, S8::kThreads, S8::kSmem, c->stream>>>(pm, c->mmaps[c->cur], c->mg,
                                                                                    it_off);
    else if (c->march_rows == 6)
      fdp::k_march<MODE, 6><<<c->march_ctas, S6::kThreads, S6::kSmem, c->stream>>>(pm, c->mmaps[c->cur], c->mg,
                                                                                    it_off);
    else
      fdp::k_march<MODE, 4><<<c->march_ctas, S4::kThreads, S4::kSmem, c->stream>>>(pm, c->mmaps[c->cur], c->mg,
                                                                                    it_off);
  }
  fdp::k_stress_frame<T, SI, MODE><<<c->nmframe_s + (defer ? mr_blocks : 0), blk, 0, c->side>>>(
      ps, (const int4*)c->mframe_s.p, c->nmframe_s, it_off, defer ? 2 : 0);
  fdp::k_velocity_frame<T, SI, MODE><<<c->nmframe_v, blk, 0, c->side>>>(pv, (const int4*)c->mframe_v.p,
                                                                          c->nmframe_v, it_off);
  if (c->core_ev[0][1]) cudaEventRecord(c->core_ev[0][1], c->stream);
  cudaEventRecord(c->join, c->side);
  cudaStreamWaitEvent(c->stream, c->join, 0);
  c->launches += 3;
  flip_buffers(c);
  if (last && edge_threads(c) > 0) {
    Params<T> pe = base;
    set_fields(c, pe, c->fields, c->fields);
    fdp::k_edge<T, SI><<<(edge_threads(c) + kBlockX - 1) / kBlockX, kBlockX, 0, c->stream>>>(pe, it_off, 1);
    c->launches += 1;
  }
}

// Level it_off of a run of levels; `first` and `last` mark the run's ends.
template <class T> int launch_level_any(fdp_ctx* c, const Params<T>& p, int it_off, bool first, bool last) {
  if (use_march(c)) {
    // the march levels run FP32 contexts only
    const bool si = c->g.stress_imaging != 0;
    switch (c->medium_mode) {
      case fdp::M_BIOT:
        if (si) launch_level_march<T, true, fdp::M_BIOT>(c, p, it_off, first, last);
        else launch_level_march<T, false, fdp::M_BIOT>(c, p, it_off, first, last);
        break;
      case fdp::M_TABLE:
        if (si) launch_level_march<T, true, fdp::M_TABLE>(c, p, it_off, first, last);
        else launch_level_march<T, false, fdp::M_TABLE>(c, p, it_off, first, last);
        break;
      default:
        if (si) launch_level_march<T, true, fdp::M_PLANES>(c, p, it_off, first, last);
        else launch_level_march<T, false, fdp::M_PLANES>(c, p, it_off, first, last);
    }
    return FDP_OK;
  }
  const bool defer = defer_edge(c);
  launch<T>(c, p, 0, it_off, defer && !first ? kDeferPrev : 0);
  launch<T>(c, p, 1, it_off, defer ? kFrameSamples : 0);
  if (edge_threads(c) > 0 && (!defer || last)) launch<T>(c, p, 2, it_off, defer ? kFrameSamples : 0);
  c->launches += fdp::edge_launch(c, it_off);  // learned absorbing edge, when attached
  return FDP_OK;
}

// Kernel launches of a run of n levels.
long long run_launches(const fdp_ctx* c, int n) {
  if (use_march(c)) return (long long)n * 3 + (edge_threads(c) > 0 ? 1 : 0);
  const int cores = c->use_core ? (!c->fused[0] && c->cs[1] > c->cs[0]) + (!c->fused[1] && c->cv[1] > c->cv[0]) : 0;
  const int edges = edge_threads(c) > 0 ? (defer_edge(c) ? 1 : n) : 0;
  return (long long)n * (2 + cores + (c->edge && c->edge_attached ? 3 : 0)) + edges;
}

// Frees every captured run of levels (their kernels' parameters changed).
void drop_graphs(fdp_ctx* c) {
  for (auto& row : c->graph)
    for (auto& g : row)
      if (g) { cudaGraphExecDestroy(g); g = nullptr; }
}

// The captured graph of a run of n levels (1 <= n <= kChunk), captured on
// first use: the run's kernels as launch_level_any enqueues them, then the
// level counter advanced by n, so a replay continues from whatever level
// *it_base holds.
template <class T> int run_graph(fdp_ctx* c, const Params<T>& p, int n, cudaGraphExec_t* out) {
  if (c->params_dirty) {
    drop_graphs(c);
    c->params_dirty = false;
  }
  cudaGraphExec_t& slot = c->graph[c->cur][n];
  if (!slot) {
    cudaGraph_t gr = nullptr;
    CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = c->launches;
    const int cur = c->cur;
    for (int k = 0; k < n; ++k) launch_level_any<T>(c, p, k, k == 0, k == n - 1);
    fdp::k_add_base<<<1, 1, 0, c->stream>>>((int*)c->itbase.p, n);
    // capture only records: the launch count and the current buffers stay
    // those before the run until the caller launches it
    c->launches = before;
    if (c->cur != cur) flip_buffers(c);
    cudaError_t e = cudaStreamEndCapture(c->stream, &gr);
    if (e != cudaSuccess) return fail(c, FDP_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&slot, gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) {
      slot = nullptr;
      return fail(c, FDP_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
    }
    // moves the graph's device-side set-up out of its first launch
    CK(c, cudaGraphUpload(slot, c->stream));
  }
  *out = slot;
  return FDP_OK;
}

// Levels it_begin..it_end: replays of the kChunk-level graph, then one
// graph of the remaining levels.  Every run length has its own graph, so a
// short run costs one graph launch, not its levels' launches one by one.
template <class T> int run_t(fdp_ctx* c, int it_begin, int it_end) {
  Params<T> p;
  fill_params<T>(c, p);
  fdp::k_set_base<<<1, 1, 0, c->stream>>>((int*)c->itbase.p, it_begin);
  c->launches += 1;
  int it = it_begin;
  while (it <= it_end) {
    const int n = std::min(kChunk, it_end - it + 1);
    cudaGraphExec_t g = nullptr;
    int rc = run_graph<T>(c, p, n, &g);
    if (rc != FDP_OK) return rc;
    CK(c, cudaGraphLaunch(g, c->stream));
    c->launches += run_launches(c, n) + 1;
    if (use_march(c) && (n & 1)) flip_buffers(c);  // the run ends in the other buffers
    it += n;
  }
  CK(c, cudaGetLastError());
  return FDP_OK;
}

// Captures the graphs a run of n_levels levels replays (fdp_prepare_run),
// for a run starting in either buffer when the levels are march levels
// (capture only records, so the buffers are swapped on the host alone).
template <class T> int prepare_t(fdp_ctx* c, int n_levels) {
  Params<T> p;
  fill_params<T>(c, p);
  cudaGraphExec_t g = nullptr;
  int rc = FDP_OK;
  const int parities = use_march(c) ? 2 : 1;
  for (int k = 0; k < parities && rc == FDP_OK; ++k) {
    if (k == 1) flip_buffers(c);
    if (n_levels >= kChunk) rc = run_graph<T>(c, p, kChunk, &g);
    if (rc == FDP_OK && n_levels % kChunk) rc = run_graph<T>(c, p, n_levels % kChunk, &g);
    if (k == 1) flip_buffers(c);
  }
  return rc;
}

// Runs fn(begin, end) over [0, n) split across the host's cores, at least
// `grain` items per thread.
template <class F> void parallel_for(size_t n, F fn, size_t grain = 65536) {
  const size_t hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const size_t nt = std::min(hw, std::max<size_t>(1, n / grain));
  if (nt <= 1) { fn((size_t)0, n); return; }
  std::vector<std::thread> th;
  for (size_t t = 0; t < nt; ++t) th.emplace_back(fn, n * t / nt, n * (t + 1) / nt);
  for (auto& x : th) x.join();
}

// A host array left uninitialised at allocation: the set-up writes every
// element it uploads from its worker threads, so a single-threaded zero
// fill of hundreds of MB (and its page faults) is not paid up front.
// Whether the n values at a have one bit pattern.
template <class T> bool same_run(const T* a, size_t n) {
  for (size_t i = 1; i < n; ++i)
    if (std::memcmp(&a[0], &a[i], sizeof(T)) != 0) return false;
  return true;
}

template <class T> struct HostBuf {
  std::unique_ptr<T[]> p;
  size_t n = 0;
  void reset(size_t m) { p.reset(new T[m]); n = m; }
  T& operator[](size_t i) { return p[i]; }
  const T& operator[](size_t i) const { return p[i]; }
  T* data() { return p.get(); }
  size_t size() const { return n; }
  // hands the memory to a thread of its own that frees it, so that the
  // caller does not wait for hundreds of megabytes to be unmapped (freed
  // here when no thread can be started)
  void release_later() {
    if (n >= ((size_t)1 << 24)) {
      try {
        std::thread([q = std::move(p)]() mutable { q.reset(); }).detach();
      } catch (...) {
      }
    }
    p.reset();
    n = 0;
  }
};

// Hashes of a column's bit patterns and of its negation's: four
// interleaved 64-bit FNV-1a lanes each (independent multiply chains),
// folded together at the end.
template <class T> void column_hash(const T* a, size_t n, uint64_t& hpos, uint64_t& hneg) {
  using U = typename std::conditional<sizeof(T) == 8, uint64_t, uint32_t>::type;
  const U sign = (U)1 << (sizeof(T) * 8 - 1);
  const uint64_t prime = 1099511628211ULL;
  uint64_t p[4], q[4];
  for (int l = 0; l < 4; ++l) p[l] = q[l] = 1469598103934665603ULL + (uint64_t)l;
  size_t i = 0;
  for (; i + 4 <= n; i += 4)
    for (int l = 0; l < 4; ++l) {
      U x;
      std::memcpy(&x, &a[i + l], sizeof(T));
      p[l] = (p[l] ^ (uint64_t)x) * prime;
      q[l] = (q[l] ^ (uint64_t)(U)(x ^ sign)) * prime;
    }
  for (; i < n; ++i) {
    U x;
    std::memcpy(&x, &a[i], sizeof(T));
    p[0] = (p[0] ^ (uint64_t)x) * prime;
    q[0] = (q[0] ^ (uint64_t)(U)(x ^ sign)) * prime;
  }
  hpos = hneg = 0;
  for (int l = 0; l < 4; ++l) {
    hpos = (hpos ^ p[l]) * prime;
    hneg = (hneg ^ q[l]) * prime;
  }
}

// The derived table of every material (column k at out[k * (jmnum+1) + j],
// index 0 unused), and per column whether it is constant and the hashes
// of its bit patterns and of their negation: materials in blocks of 65536,
// derived and hashed block by block in parallel while the block is in
// cache, the blocks' hashes combined in block order.
template <class T>
void derive_table(const int32_t jmnum, const T* tab, HostBuf<T>& out, bool* constant, uint64_t* hpos,
                  uint64_t* hneg) {
  // table24 columns (.MO record order, read_model_par.F90:52-60)
  enum { MU, SXX1, SXX2, SXX3, SZZ1, SZZ2, SZZ3, P1, P2, P3, R1U, R1W, R2U, R2W, R3U, R3W,
         R1QX, R1QZ, R2QX, R2QZ, R3QX, R3QZ, AUXW, AUXQZ };
  const size_t ld = (size_t)jmnum + 1;
  out.reset(ld * fdp::C_NCOEF);
  for (int k = 0; k < fdp::C_NCOEF; ++k) out[(size_t)k * ld] = T(0);  // index 0: no material
  constexpr size_t kBlk = 65536;
  constexpr int NC = fdp::C_NCOEF;
  const size_t nblk = ((size_t)jmnum + kBlk - 1) / kBlk;
  std::vector<uint64_t> bp(nblk * NC), bn(nblk * NC);
  std::vector<char> bconst(nblk * NC);
  using U = typename std::conditional<sizeof(T) == 8, uint64_t, uint32_t>::type;
  std::vector<U> bfirst(nblk * NC);
  parallel_for(nblk, [&](size_t b0, size_t b1) {
  for (size_t blk = b0; blk < b1; ++blk) {
  const int jb = (int)(blk * kBlk), je = (int)std::min((size_t)jmnum, (blk + 1) * kBlk);
  for (int j = jb + 1; j <= je; ++j) {
    const T* r = tab + (size_t)(j - 1) * 24;
    auto put = [&](int k, T v) { out[(size_t)k * ld + j] = v; };
    put(fdp::C_MU, r[MU]);
    put(fdp::C_SXX1, r[SXX1]); put(fdp::C_SXX2, r[SXX2]); put(fdp::C_SXX3, r[SXX3]);
    put(fdp::C_SZZ1, r[SZZ1]); put(fdp::C_SZZ2, r[SZZ2]); put(fdp::C_SZZ3, r[SZZ3]);
    put(fdp::C_P1, r[P1]); put(fdp::C_P2, r[P2]); put(fdp::C_P3, r[P3]);
    // inh_qx_int.F90:44 and inh_v_uv_int.F90:46, evaluated per material
    // each exponential evaluated once (the same call gives the same value)
    const T eqx = std::exp(-r[R3QX]), eqz = std::exp(-r[R3QZ]);
    put(fdp::C_EQX, eqx);
    put(fdp::C_CU, (r[R2U] / r[R3QX]) * (T(1) - eqx));
    put(fdp::C_R1QX, r[R1QX]); put(fdp::C_R2QX, r[R2QX]);
    put(fdp::C_R1U, r[R1U]); put(fdp::C_R3U, r[R3U]);
    put(fdp::C_EQZ, eqz);
    put(fdp::C_CW, (r[R2W] / r[R3QZ]) * (T(1) - eqz));
    put(fdp::C_R1QZ, r[R1QZ]); put(fdp::C_R2QZ, r[R2QZ]);
    put(fdp::C_R1W, r[R1W]); put(fdp::C_R3W, r[R3W]);
    put(fdp::C_AUXW, r[AUXW]); put(fdp::C_AUXQZ, r[AUXQZ]);
  }
  for (int k = 0; k < NC; ++k) {
    const T* col = &out[(size_t)k * ld + jb + 1];
    const size_t n = (size_t)(je - jb);
    column_hash(col, n, bp[blk * NC + k], bn[blk * NC + k]);
    U f;
    std::memcpy(&f, col, sizeof(T));
    bfirst[blk * NC + k] = f;
    bconst[blk * NC + k] = same_run(col, n);
  }
  }
  }, 1);
  const uint64_t prime = 1099511628211ULL;
  for (int k = 0; k < NC; ++k) {
    uint64_t p = 1469598103934665603ULL, q = p;
    bool cst = true;
    for (size_t blk = 0; blk < nblk; ++blk) {
      p = (p ^ bp[blk * NC + k]) * prime;
      q = (q ^ bn[blk * NC + k]) * prime;
      cst = cst && bconst[blk * NC + k] && bfirst[blk * NC + k] == bfirst[k];
    }
    hpos[k] = p;
    hneg[k] = q;
    constant[k] = cst;
  }
}

// Materials at most this many use table mode when some coefficient varies;
// a larger table (one material per cell) is expanded into per-cell planes.
constexpr int kMaxTableMaterials = 4096;

template <class T> bool same_bits(const T* a, const T* b, size_t n, bool negate);

// same_bits over many elements, split across the host's cores.
template <class T> bool same_bits_par(const T* a, const T* b, size_t n, bool negate) {
  std::atomic<bool> same{true};
  parallel_for(n, [&](size_t lo, size_t hi) {
    if (!same_bits(a + lo, b + lo, hi - lo, negate)) same = false;
  });
  return same;
}

template <class T> bool same_bits(const T* a, const T* b, size_t n, bool negate) {
  using U = typename std::conditional<sizeof(T) == 8, uint64_t, uint32_t>::type;
  const U sign = (U)1 << (sizeof(T) * 8 - 1);
  for (size_t i = 0; i < n; ++i) {
    U x, y;
    std::memcpy(&x, &a[i], sizeof(T));
    std::memcpy(&y, &b[i], sizeof(T));
    if ((negate ? (x ^ sign) : x) != y) return false;
  }
  return true;
}

// Chooses the device representation of the medium and uploads it: the
// derived coefficient columns are classified as constant (folded into the
// kernel parameters), equal up to sign to an earlier column (shared plane),
// or distinct; distinct columns become per-cell planes when the material
// table is large, else the kernels index the table through JM.
template <class T> int build_medium(fdp_ctx* c, const int32_t* jm, int32_t jmnum, const T* table24) {
  HostBuf<T> t;
  bool constant[fdp::C_NCOEF];
  uint64_t hpos[fdp::C_NCOEF], hneg[fdp::C_NCOEF];
  derive_table<T>(jmnum, table24, t, constant, hpos, hneg);
  const size_t ld = (size_t)jmnum + 1;
  int rc;
  // AUXIL_W / AUXIL_QZ of JM(I,0) (inh_w_qz_int_1_si.F90:32)
  std::vector<T> aux((size_t)2 * c->NX);
  for (int x = 0; x < c->NX; ++x) {
    const int j = jm[x];
    aux[x] = t[(size_t)fdp::C_AUXW * ld + j];
    aux[(size_t)c->NX + x] = t[(size_t)fdp::C_AUXQZ * ld + j];
  }
  if ((rc = dev_alloc(c, c->aux, aux.size() * sizeof(T))) != FDP_OK) return rc;
  if ((rc = copy_sync(c, c->aux.p, aux.data(), aux.size() * sizeof(T), cudaMemcpyHostToDevice)) != FDP_OK) return rc;
  // column classification (the AUXIL columns are served by `aux` above):
  // constant columns and the hashes of every column and of its negation
  // come with the derived table; a hash match is confirmed by comparing
  // every bit
  // plane assignment: first on the hashes alone, then every column placed
  // on an earlier plane is confirmed bit for bit in one parallel pass; a
  // failed confirmation (a hash collision) redoes the assignment with a
  // full comparison before each match
  std::vector<int> plane_col;
  auto assign = [&](bool exact) {
    plane_col.clear();
    for (int k = 0; k < fdp::C_NCOEF; ++k) {
      c->src[k] = -1; c->neg[k] = 0; c->cval_d[k] = 0; c->cval_f[k] = 0;
      if (k == fdp::C_AUXW || k == fdp::C_AUXQZ) continue;
      const T* col = &t[(size_t)k * ld + 1];
      if (constant[k]) {
        c->cval_d[k] = (double)col[0];
        c->cval_f[k] = (float)col[0];
        continue;
      }
      for (size_t q = 0; q < plane_col.size() && c->src[k] < 0; ++q) {
        const int o = plane_col[q];
        const T* other = &t[(size_t)o * ld + 1];
        if (hpos[o] == hpos[k] && (!exact || same_bits_par(other, col, (size_t)jmnum, false))) {
          c->src[k] = (int)q; c->neg[k] = 0;
        } else if (hpos[o] == hneg[k] && (!exact || same_bits_par(other, col, (size_t)jmnum, true))) {
          c->src[k] = (int)q; c->neg[k] = 1;
        }
      }
      if (c->src[k] < 0) { c->src[k] = (int)plane_col.size(); plane_col.push_back(k); }
    }
  };
  assign(false);
  {
    std::vector<int> alias;  // columns placed on another column's plane
    for (int k = 0; k < fdp::C_NCOEF; ++k)
      if (c->src[k] >= 0 && plane_col[c->src[k]] != k) alias.push_back(k);
    std::atomic<bool> same{true};
    if (!alias.empty())
      parallel_for((size_t)jmnum, [&](size_t lo, size_t hi) {
        for (int k : alias) {
          const T* col = &t[(size_t)k * ld + 1 + lo];
          const T* other = &t[(size_t)plane_col[c->src[k]] * ld + 1 + lo];
          if (!same_bits(other, col, hi - lo, c->neg[k] != 0)) { same = false; return; }
        }
      });
    if (!same) assign(true);
  }
  c->nplanes = (int)plane_col.size();
  const bool table_mode = c->nplanes > 0 && jmnum <= kMaxTableMaterials;
  // Biot relations: ten distinct planes, in first-occurrence order equal to
  // the slot order, and every column on its slot with its sign
  bool biot = !table_mode && c->nplanes == 10;
  for (int k = 0; k < fdp::C_AUXW && biot; ++k)
    biot = c->src[k] == fdp::biot_slot(k) && (c->neg[k] != 0) == fdp::biot_neg(k);
  c->medium_mode = table_mode ? fdp::M_TABLE : biot ? fdp::M_BIOT : fdp::M_PLANES;
  const size_t cells = (size_t)c->rows_alloc * c->pitch;
  if (table_mode) {
    // JM into the padded field layout (padding holds material 1) and the table
    std::vector<int32_t> h(cells, 1);
    for (int L = 0; L < c->NZ; ++L)
      std::memcpy(&h[(size_t)(L + kPadZ) * c->pitch + kPadX], jm + (size_t)L * c->NX, (size_t)c->NX * sizeof(int32_t));
    if ((rc = dev_alloc(c, c->jm, h.size() * sizeof(int32_t))) != FDP_OK) return rc;
    if ((rc = copy_sync(c, c->jm.p, h.data(), h.size() * sizeof(int32_t), cudaMemcpyHostToDevice)) != FDP_OK) return rc;
    if ((rc = dev_alloc(c, c->coef, t.size() * sizeof(T))) != FDP_OK) return rc;
    if ((rc = copy_sync(c, c->coef.p, t.data(), t.size() * sizeof(T), cudaMemcpyHostToDevice)) != FDP_OK) return rc;
    dev_alloc(c, c->planes, 0);
  } else {
    dev_alloc(c, c->jm, 0);
    dev_alloc(c, c->coef, 0);
    if ((rc = dev_alloc(c, c->planes, std::max<size_t>(1, (size_t)c->nplanes * cells) * sizeof(T))) != FDP_OK) return rc;
    // every plane expanded over the padded layout (padding holds material
    // 1), rows in parallel, then one copy
    HostBuf<T> pl;
    pl.reset((size_t)c->nplanes * cells);
    parallel_for((size_t)c->nplanes * c->rows_alloc, [&](size_t b, size_t e) {
      for (size_t r = b; r < e; ++r) {
        const int q = (int)(r / c->rows_alloc), row = (int)(r % c->rows_alloc);
        const T* col = &t[(size_t)plane_col[q] * ld];
        T* dst = &pl[(size_t)q * cells + (size_t)row * c->pitch];
        const int L = row - kPadZ;
        if (L < 0 || L >= c->NZ) { std::fill(dst, dst + c->pitch, col[1]); continue; }
        std::fill(dst, dst + kPadX, col[1]);
        const int32_t* src = jm + (size_t)L * c->NX;
        for (int x = 0; x < c->NX; ++x) dst[kPadX + x] = col[src[x]];
        std::fill(dst + kPadX + c->NX, dst + c->pitch, col[1]);
      }
    }, 16);
    if ((rc = copy_sync(c, c->planes.p, pl.data(), pl.size() * sizeof(T), cudaMemcpyHostToDevice)) != FDP_OK) return rc;
    pl.release_later();
  }
  t.release_later();
  return FDP_OK;
}

}  // namespace

extern "C" {

int fdp_create(const fdp_grid* g, fdp_ctx** out) {
  const TraceRange trace("fdp_create");
  if (!g || !out) return fail(nullptr, FDP_ERR_ARG, "null argument");
  *out = nullptr;
  if (g->precision != FDP_F32 && g->precision != FDP_F64)
    return fail(nullptr, FDP_ERR_ARG, "precision must be FDP_F32 or FDP_F64");
  if (g->mx < 8 || g->mz < 8 || g->tpml < 0)
    return fail(nullptr, FDP_ERR_ARG, "need MX >= 8, MZ >= 8, TPML >= 0 (got %d, %d, %d)", g->mx, g->mz, g->tpml);
  // The reference updates the source row with HPLANE_LIN_STRESS in addition
  // to the row's own routine when LIN_Z lies outside the interior rows
  // (time_loop.F90:93-124): such a source row is rejected.
  if (g->lin_z < 2 || g->lin_z > g->mz - 2)
    return fail(nullptr, FDP_ERR_ARG, "source row LIN_Z=%d must lie in 2..MZ-2=%d", g->lin_z, g->mz - 2);
  if (!(g->h > 0) || !(g->dt > 0)) return fail(nullptr, FDP_ERR_ARG, "H and DT must be positive");
  fdp_ctx* c = new fdp_ctx();
  c->g = *g;
  c->prec = g->precision;
  c->MX = g->mx; c->MZ = g->mz; c->TPML = g->tpml;
  c->MX1 = c->MX - 1;
  c->PMLL = 1 - c->TPML; c->PMLXH = c->MX + c->TPML; c->PMLZH = c->MZ + c->TPML;
  c->NX = c->PMLXH - c->PMLL + 1;
  c->NZ = c->PMLZH + 1;
  c->pitch = ((c->NX + 2 * kPadX + 31) / 32) * 32;
  c->rows_alloc = c->NZ + 2 * kPadZ;
  auto bail = [&](int code) { g_create_error = c->err; fdp_destroy(c); return code; };
  cudaError_t e = cudaSetDevice(g->device);
  if (e != cudaSuccess) { c->err = std::string("cudaSetDevice: ") + cudaGetErrorString(e); return bail(FDP_ERR_CUDA); }
  e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) { c->err = std::string("cudaStreamCreate: ") + cudaGetErrorString(e); return bail(FDP_ERR_CUDA); }
  const size_t es = (size_t)c->prec;
  const size_t fbytes = (size_t)c->rows_alloc * c->pitch * es;
  int rc;
  for (int k = 0; k < 8; ++k)
    if ((rc = dev_alloc(c, c->fields[k], fbytes)) != FDP_OK) return bail(rc);
  if ((rc = dev_alloc(c, c->jm, (size_t)c->rows_alloc * c->pitch * sizeof(int32_t))) != FDP_OK) return bail(rc);
  const int TP = c->TPML;
  const size_t pshape[24] = {
      (size_t)(TP + 1) * c->NZ, (size_t)(TP + 1) * c->NZ, (size_t)(TP + 1) * c->NZ, (size_t)(TP + 1) * c->NZ,
      (size_t)(TP + 1) * c->NZ, (size_t)(TP + 1) * c->NZ, (size_t)(TP + 1) * c->NZ, (size_t)(TP + 1) * c->NZ,
      (size_t)(TP + 1) * c->NX, (size_t)(TP + 1) * c->NX, (size_t)(TP + 1) * c->NX, (size_t)(TP + 1) * c->NX,
      (size_t)(TP + 2) * c->NZ, (size_t)(TP + 2) * c->NZ, (size_t)(TP + 2) * c->NZ, (size_t)(TP + 2) * c->NZ,
      (size_t)(TP + 2) * c->NZ, (size_t)(TP + 2) * c->NZ, (size_t)(TP + 2) * c->NZ, (size_t)(TP + 2) * c->NZ,
      (size_t)(TP + 2) * c->NX, (size_t)(TP + 2) * c->NX, (size_t)(TP + 2) * c->NX, (size_t)(TP + 2) * c->NX};
  for (int k = 0; k < 24; ++k)
    if ((rc = dev_alloc(c, c->prof[k], pshape[k] * es)) != FDP_OK) return bail(rc);
  for (int k = 0; k < 27; ++k) {
    int b[4];
    bounds_of(c, FDP_PZXL + k, b);
    if ((rc = dev_alloc(c, c->mem[k], count_of(b) * es)) != FDP_OK) return bail(rc);
  }
  if ((rc = dev_alloc(c, c->ab, 16 * es)) != FDP_OK) return bail(rc);
  if ((rc = dev_alloc(c, c->hist, (size_t)12 * c->NX * es)) != FDP_OK) return bail(rc);
  if ((rc = dev_alloc(c, c->itbase, sizeof(int))) != FDP_OK) return bail(rc);
  if ((rc = dev_alloc(c, c->errbuf, sizeof(int))) != FDP_OK) return bail(rc);
  const char* variant = std::getenv("FDP_KERNEL_VARIANT");
  c->use_tma = variant && std::strcmp(variant, "tma") == 0;
  c->use_core = !(variant && (std::strcmp(variant, "tma") == 0 || std::strcmp(variant, "global") == 0));
  // frame and core on two streams; "fused" puts each phase's frame units
  // among its core blocks in one launch instead (measured on the layered
  // 2048^2 workload: a level takes 0.1085 ms split, 0.121 ms fused, 0.1105
  // ms with only the velocity phase fused)
  const bool fused = variant && std::strcmp(variant, "fused") == 0;
  c->fused[0] = c->use_core && fused;
  c->fused[1] = c->use_core && fused;
  c->core_tma_req = c->use_core && variant && std::strcmp(variant, "coretma") == 0;
  // march levels unless a variant is named ("split" or "core": the
  // frame/core split alone); plan_core and the medium decide whether they run
  c->march_forced = variant && std::strcmp(variant, "march") == 0;
  c->march = c->use_core && (!variant || !*variant || c->march_forced);
  if (c->use_core) {
    if ((rc = plan_core(c)) != FDP_OK) return bail(rc);
    e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming);

    if (e != cudaSuccess) { c->err = std::string("side stream: ") + cudaGetErrorString(e); return bail(FDP_ERR_CUDA); }
  }
  if (c->use_tma) {
    for (int k = 0; k < 4; ++k) {
      if ((rc = make_field_map(c, &c->tma_vel.m[k], c->fields[k].p)) != FDP_OK) return bail(rc);
      if ((rc = make_field_map(c, &c->tma_str.m[k], c->fields[4 + k].p)) != FDP_OK) return bail(rc);
    }
  }
  e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) { c->err = std::string("init: ") + cudaGetErrorString(e); return bail(FDP_ERR_CUDA); }
  *out = c;
  return FDP_OK;
}

// Lets go of a shared medium: the arrays stay with the share (freed by its
// last holder) and this context's handles are cleared.
void unshare_medium(fdp_ctx* c) {
  if (!c->medium_share) return;
  c->jm = DevArr{}; c->coef = DevArr{}; c->planes = DevArr{}; c->aux = DevArr{};
  c->medium_share.reset();
}

int fdp_set_medium(fdp_ctx* c, const int32_t* jm, int32_t nx, int32_t nz, int32_t jmnum, const void* table24) {
  const TraceRange trace("fdp_set_medium");
  if (!c || !jm || !table24) return fail(c, FDP_ERR_ARG, "null argument");
  if (nx != c->NX || nz != c->NZ) return fail(c, FDP_ERR_ARG, "JM is %dx%d, grid is %dx%d", nx, nz, c->NX, c->NZ);
  if (jmnum < 1) return fail(c, FDP_ERR_ARG, "JMNUM must be >= 1");
  std::atomic<size_t> bad{(size_t)-1};
  parallel_for((size_t)nx * nz, [&](size_t lo, size_t hi) {
    for (size_t k = lo; k < hi; ++k)
      if (jm[k] < 1 || jm[k] > jmnum) {
        size_t cur = bad.load();
        while (k < cur && !bad.compare_exchange_weak(cur, k)) {}
        break;
      }
  });
  if (bad.load() != (size_t)-1) {
    const size_t k = bad.load();
    return fail(c, FDP_ERR_ARG, "JM value %d at %zu outside 1..%d", jm[k], k, jmnum);
  }
  int rc;
  CK(c, cudaStreamSynchronize(c->stream));
  unshare_medium(c);
  // host scratch of the size of the grid: a failed allocation is an error
  // code, not an exception across the ABI
  try {
    rc = (c->prec == 8) ? build_medium<double>(c, jm, jmnum, (const double*)table24)
                        : build_medium<float>(c, jm, jmnum, (const float*)table24);
  } catch (const std::bad_alloc&) {
    return fail(c, FDP_ERR_ALLOC, "host memory for the medium's set-up");
  }
  if (rc != FDP_OK) return rc;
  CK(c, cudaStreamSynchronize(c->stream));
  if ((rc = make_core_maps(c)) != FDP_OK) return rc;
  if ((rc = make_march_maps(c)) != FDP_OK) return rc;
  c->jmnum = jmnum;
  c->have_medium = true;
  params_changed(c);
  return FDP_OK;
}

int fdp_share_medium(fdp_ctx* dst, fdp_ctx* src) {
  const TraceRange trace("fdp_share_medium");
  if (!dst || !src) return fail(dst, FDP_ERR_ARG, "null argument");
  if (dst == src) return FDP_OK;
  if (!src->have_medium) return fail(dst, FDP_ERR_STATE, "the source context has no medium yet");
  if (dst->prec != src->prec || dst->NX != src->NX || dst->NZ != src->NZ || dst->g.device != src->g.device)
    return fail(dst, FDP_ERR_ARG, "a medium is shared only between contexts of the same grid, precision and device");
  CK(dst, cudaStreamSynchronize(dst->stream));  // work that may still read dst's own medium
  CK(dst, cudaStreamSynchronize(src->stream));
  if (!src->medium_share) {
    // the source's arrays move into a share; its handles stay valid
    src->medium_share = std::make_shared<MediumShare>();
    src->medium_share->jm = src->jm; src->medium_share->coef = src->coef;
    src->medium_share->planes = src->planes; src->medium_share->aux = src->aux;
  }
  unshare_medium(dst);
  int rc;
  for (DevArr* a : {&dst->jm, &dst->coef, &dst->planes, &dst->aux})
    if ((rc = dev_alloc(dst, *a, 0)) != FDP_OK) return rc;
  dst->jm = src->jm; dst->coef = src->coef; dst->planes = src->planes; dst->aux = src->aux;
  dst->medium_share = src->medium_share;
  dst->medium_mode = src->medium_mode;
  dst->nplanes = src->nplanes;
  for (int k = 0; k < fdp::C_NCOEF; ++k) {
    dst->src[k] = src->src[k]; dst->neg[k] = src->neg[k];
    dst->cval_d[k] = src->cval_d[k]; dst->cval_f[k] = src->cval_f[k];
  }
  dst->jmnum = src->jmnum;
  dst->have_medium = true;
  params_changed(dst);
  if ((rc = make_core_maps(dst)) != FDP_OK) return rc;
  return make_march_maps(dst);
}

int fdp_set_pml(fdp_ctx* c, const void* const* prof) {
  if (!c || !prof) return fail(c, FDP_ERR_ARG, "null argument");
  const size_t es = (size_t)c->prec;
  int rc;
  CK(c, cudaStreamSynchronize(c->stream));
  for (int k = 0; k < 24; ++k) {
    if (!prof[k]) return fail(c, FDP_ERR_ARG, "profile %d is null", k);
    const bool zprof = (k >= 8 && k < 12) || k >= 20;
    if (!zprof) {
      if ((rc = copy_sync(c, c->prof[k].p, prof[k], c->prof[k].bytes, cudaMemcpyHostToDevice)) != FDP_OK) return rc;
    } else {
      // (0:nj-1, PMLL:PMLXH) -> [J][I-PMLL]
      const int nj = (k < 12) ? c->TPML + 1 : c->TPML + 2;
      std::vector<unsigned char> t(c->prof[k].bytes);
      const unsigned char* s = (const unsigned char*)prof[k];
      for (int i = 0; i < c->NX; ++i)
        for (int j = 0; j < nj; ++j)
          std::memcpy(&t[((size_t)j * c->NX + i) * es], &s[((size_t)i * nj + j) * es], es);
      if ((rc = copy_sync(c, c->prof[k].p, t.data(), t.size(), cudaMemcpyHostToDevice)) != FDP_OK) return rc;
    }
  }
  c->have_pml = true;
  return FDP_OK;
}

int fdp_set_pml_arrays(fdp_ctx* c, const void* oda_xl, const void* odb_xl, const void* odc_xl, const void* odd_xl,
                       const void* oda_xh, const void* odb_xh, const void* odc_xh, const void* odd_xh,
                       const void* oda_zh, const void* odb_zh, const void* odc_zh, const void* odd_zh,
                       const void* oda2_xl, const void* odb2_xl, const void* odc2_xl, const void* odd2_xl,
                       const void* oda2_xh, const void* odb2_xh, const void* odc2_xh, const void* odd2_xh,
                       const void* oda2_zh, const void* odb2_zh, const void* odc2_zh, const void* odd2_zh) {
  const void* const prof[24] = {oda_xl,  odb_xl,  odc_xl,  odd_xl,  oda_xh,  odb_xh,  odc_xh,  odd_xh,
                                oda_zh,  odb_zh,  odc_zh,  odd_zh,  oda2_xl, odb2_xl, odc2_xl, odd2_xl,
                                oda2_xh, odb2_xh, odc2_xh, odd2_xh, oda2_zh, odb2_zh, odc2_zh, odd2_zh};
  return fdp_set_pml(c, prof);
}

int fdp_set_bottom_nr(fdp_ctx* c, const void* ab16) {
  if (!c || !ab16) return fail(c, FDP_ERR_ARG, "null argument");
  int rc;
  CK(c, cudaStreamSynchronize(c->stream));
  if ((rc = copy_sync(c, c->ab.p, ab16, 16 * (size_t)c->prec, cudaMemcpyHostToDevice)) != FDP_OK) return rc;
  c->have_nr = true;
  return FDP_OK;
}

int fdp_set_source(fdp_ctx* c, const void* sourtf, int32_t mt2) {
  if (!c || !sourtf) return fail(c, FDP_ERR_ARG, "null argument");
  if (mt2 < 1) return fail(c, FDP_ERR_ARG, "MT2 must be >= 1");
  CK(c, cudaStreamSynchronize(c->stream));
  int rc;
  if ((rc = dev_alloc(c, c->stf, (size_t)2 * mt2 * c->prec)) != FDP_OK) return rc;
  if ((rc = copy_sync(c, c->stf.p, sourtf, (size_t)2 * mt2 * c->prec, cudaMemcpyHostToDevice)) != FDP_OK) return rc;
  c->mt2 = mt2;
  c->have_source = true;
  params_changed(c);
  if (c->mr > 0) {
    if ((rc = dev_alloc(c, c->raw, (size_t)c->mt2 * c->mr * 6 * c->prec)) != FDP_OK) return rc;
  }
  CK(c, cudaStreamSynchronize(c->stream));
  return FDP_OK;
}

int fdp_set_receivers(fdp_ctx* c, const int32_t* irecx, const int32_t* lrecx, const int32_t* irecz,
                      const int32_t* lrecz, int32_t mr, int32_t flags) {
  if (!c) return fail(c, FDP_ERR_ARG, "null context");
  if (mr < 0 || (mr > 0 && (!irecx || !lrecx || !irecz || !lrecz))) return fail(c, FDP_ERR_ARG, "bad receiver arrays");
  CK(c, cudaStreamSynchronize(c->stream));
  std::vector<int32_t> r((size_t)4 * mr);
  for (int j = 0; j < mr; ++j) { r[4 * j] = irecx[j]; r[4 * j + 1] = lrecx[j]; r[4 * j + 2] = irecz[j]; r[4 * j + 3] = lrecz[j]; }
  int rc;
  if ((rc = dev_alloc(c, c->rec, r.size() * sizeof(int32_t))) != FDP_OK) return rc;
  if (mr > 0) if ((rc = copy_sync(c, c->rec.p, r.data(), r.size() * sizeof(int32_t), cudaMemcpyHostToDevice)) != FDP_OK) return rc;
  c->mr = mr;
  c->rec_flags = flags;
  if (c->mt2 > 0 && mr > 0) {
    if ((rc = dev_alloc(c, c->raw, (size_t)c->mt2 * mr * 6 * c->prec)) != FDP_OK) return rc;
  }
  CK(c, cudaStreamSynchronize(c->stream));
  params_changed(c);
  return FDP_OK;
}

int fdp_run(fdp_ctx* c, int32_t it_begin, int32_t it_end) {
  const TraceRange trace("fdp_run");
  if (!c) return fail(c, FDP_ERR_ARG, "null context");
  if (!c->have_medium || !c->have_pml || !c->have_nr || !c->have_source)
    return fail(c, FDP_ERR_STATE, "set medium, PML profiles, bottom coefficients and source before fdp_run");
  if (it_begin < 1 || it_end > c->mt2 || it_end < it_begin - 1)
    return fail(c, FDP_ERR_ARG, "levels %d..%d outside 1..MT2=%d", it_begin, it_end, c->mt2);
  if (c->mr > 0 && !c->raw.p) return fail(c, FDP_ERR_STATE, "receiver buffer missing");
  if (it_end < it_begin) return FDP_OK;
  CK(c, cudaSetDevice(c->g.device));
  int rc = (c->prec == 8) ? run_t<double>(c, it_begin, it_end) : run_t<float>(c, it_begin, it_end);
  if (rc == FDP_OK && it_end > c->last_it) c->last_it = it_end;
  return rc;
}

int fdp_prepare_run(fdp_ctx* c, int32_t n_levels) {
  const TraceRange trace("fdp_prepare_run");
  if (!c) return fail(c, FDP_ERR_ARG, "null context");
  if (!c->have_medium || !c->have_pml || !c->have_nr || !c->have_source)
    return fail(c, FDP_ERR_STATE, "set medium, PML profiles, bottom coefficients and source before fdp_prepare_run");
  if (n_levels < 0) return fail(c, FDP_ERR_ARG, "negative number of levels");
  if (c->mr > 0 && !c->raw.p) return fail(c, FDP_ERR_STATE, "receiver buffer missing");
  if (n_levels == 0) return FDP_OK;
  CK(c, cudaSetDevice(c->g.device));
  return (c->prec == 8) ? prepare_t<double>(c, n_levels) : prepare_t<float>(c, n_levels);
}

int fdp_get_receivers(fdp_ctx* c, int32_t it_first, int32_t n_levels, void* host) {
  const TraceRange trace("fdp_get_receivers");
  if (!c || (!host && n_levels > 0)) return fail(c, FDP_ERR_ARG, "null argument");
  if (n_levels <= 0 || c->mr == 0) return FDP_OK;
  if (it_first < 1 || it_first + n_levels - 1 > c->mt2) return fail(c, FDP_ERR_ARG, "levels outside 1..MT2");
  if (int rc = device_status(c)) return rc;
  const int mr = c->mr;
  const int lo = it_first - 1;  // also fetch the previous level for the time derivative
  const int first_fetch = std::max(lo, 1);
  const int nfetch = it_first + n_levels - first_fetch;
  const size_t lev = (size_t)mr * 6;
  auto body = [&](auto zero) -> int {
    using T = decltype(zero);
    HostBuf<T> raw;
    raw.reset((size_t)nfetch * lev);
    int rc = copy_sync(c, raw.data(), (const T*)c->raw.p + (size_t)(first_fetch - 1) * lev,
                       raw.size() * sizeof(T), cudaMemcpyDeviceToHost);
    if (rc != FDP_OK) return rc;
    const T DT = (T)c->g.dt;
    T* out = (T*)host;
    // levels in parallel (each level's values depend on its own and the
    // previous level's samples only)
    parallel_for((size_t)n_levels, [&](size_t nb, size_t ne) {
    for (int n = (int)nb; n < (int)ne; ++n) {
      const int it = it_first + n;
      const T* cur = &raw[(size_t)(it - first_fetch) * lev];
      const T* prv = (it - 1 >= first_fetch) ? &raw[(size_t)(it - 1 - first_fetch) * lev] : nullptr;
      for (int j = 0; j < mr; ++j) {
        T* r = out + ((size_t)n * mr + j) * FDP_REC_VALUES;
        const T* s = cur + (size_t)j * 6;
        const T* q = prv ? prv + (size_t)j * 6 : nullptr;
        auto prev = [&](int k) { return q ? q[k] : T(0); };
        for (int k = 0; k < FDP_REC_VALUES; ++k) r[k] = T(0);
        if (c->rec_flags & FDP_REC_TLV) {
          // store_seismograms.F90:65-66,92-93: SPU=(S-SSU)/DT, SSU=S
          r[0] = s[0]; r[1] = s[1];
          r[2] = (s[0] - prev(0)) / DT; r[3] = (s[1] - prev(1)) / DT;
          if (c->rec_flags & FDP_REC_TLQ) {
            r[4] = s[2]; r[5] = s[3];
            r[6] = (s[2] - prev(2)) / DT; r[7] = (s[3] - prev(3)) / DT;
          }
        }
        if (c->rec_flags & FDP_REC_TLP) { r[8] = s[4]; r[9] = s[5]; }
      }
    }
    }, 64);
    raw.release_later();
    return FDP_OK;
  };
  try {
    return c->prec == 8 ? body(0.0) : body(0.0f);
  } catch (const std::bad_alloc&) {
    return fail(c, FDP_ERR_ALLOC, "host memory for the receiver samples");
  }
}

int fdp_field_bounds(fdp_ctx* c, int32_t id, int32_t* b4) {
  if (!c || !b4) return fail(c, FDP_ERR_ARG, "null argument");
  int b[4];
  if (!bounds_of(c, id, b)) return fail(c, FDP_ERR_ARG, "unknown field id %d", id);
  for (int k = 0; k < 4; ++k) b4[k] = b[k];
  return FDP_OK;
}

static int field_copy(fdp_ctx* c, int32_t id, void* host, bool set) {
  if (!c || !host) return fail(c, FDP_ERR_ARG, "null argument");
  int b[4];
  if (!bounds_of(c, id, b)) return fail(c, FDP_ERR_ARG, "unknown field id %d", id);
  if (id == FDP_QXP || id == FDP_QZP) return fail(c, FDP_ERR_UNSUPPORTED, "QXP/QZP are not stored by this engine");
  if (int rc = device_status(c)) return rc;
  const size_t es = (size_t)c->prec;
  if (id <= FDP_PRES) {
    char* dev = (char*)c->fields[id].p + ((size_t)kPadZ * c->pitch + kPadX) * es;
    if (set && c->alt[id].p) {
      // both buffers: cells no level updates are read from either
      char* dev2 = (char*)c->alt[id].p + ((size_t)kPadZ * c->pitch + kPadX) * es;
      int rc = copy2d_sync(c, dev2, c->pitch * es, host, c->NX * es, c->NX * es, c->NZ, cudaMemcpyHostToDevice);
      if (rc != FDP_OK) return rc;
    }
    if (set)
      return copy2d_sync(c, dev, c->pitch * es, host, c->NX * es, c->NX * es, c->NZ, cudaMemcpyHostToDevice);
    else
      return copy2d_sync(c, host, c->NX * es, dev, c->pitch * es, c->NX * es, c->NZ, cudaMemcpyDeviceToHost);
    return FDP_OK;
  }
  void* dev;
  if (id >= FDP_SZ_U) dev = (char*)c->hist.p + (size_t)(id - FDP_SZ_U) * 3 * c->NX * es;
  else dev = c->mem[id - FDP_PZXL].p;
  const size_t n = count_of(b) * es;
  if (set) return copy_sync(c, dev, host, n, cudaMemcpyHostToDevice);
  return copy_sync(c, host, dev, n, cudaMemcpyDeviceToHost);
}

int fdp_get_field(fdp_ctx* c, int32_t id, void* host) { return field_copy(c, id, host, false); }
int fdp_set_field(fdp_ctx* c, int32_t id, const void* host) { return field_copy(c, id, (void*)host, true); }

int fdp_get_snapshot(fdp_ctx* c, int32_t mask, void* host) {
  if (!c || !host) return fail(c, FDP_ERR_ARG, "null argument");
  const size_t n = (size_t)c->NX * c->NZ * c->prec;
  char* out = (char*)host;
  const int ids[4] = {FDP_UM, FDP_WM, FDP_QX, FDP_QZ};
  for (int k = 0; k < 4; ++k) {
    if (!(mask & (1 << k))) continue;
    int rc = field_copy(c, ids[k], out, false);
    if (rc != FDP_OK) return rc;
    out += n;
  }
  return FDP_OK;
}

int fdp_synchronize(fdp_ctx* c) {
  if (!c) return fail(c, FDP_ERR_ARG, "null context");
  return device_status(c);
}

int fdp_diag_wait_timeout(fdp_ctx* c, int32_t polls) {
  if (!c || polls < 1 || polls > (1 << 20)) return fail(c, FDP_ERR_ARG, "need a context and 1..2^20 polls");
  int rc;
  if (!c->diag_flag.p && (rc = dev_alloc(c, c->diag_flag, sizeof(int))) != FDP_OK) return rc;
  fdp::k_wait_flag<<<1, 1, 0, c->stream>>>((const int*)c->diag_flag.p, (unsigned)polls, (int*)c->errbuf.p);
  c->launches += 1;
  CK(c, cudaGetLastError());
  return FDP_OK;
}

int64_t fdp_kernel_launches(fdp_ctx* c) { return c ? c->launches : 0; }

int fdp_medium_info(fdp_ctx* c, int32_t* mode, int32_t* planes_stress, int32_t* planes_velocity) {
  if (!c || !mode || !planes_stress || !planes_velocity) return fail(c, FDP_ERR_ARG, "null argument");
  if (!c->have_medium) return fail(c, FDP_ERR_STATE, "no medium set");
  auto count = [&](int k0, int k1) {
    bool seen[fdp::C_NCOEF] = {};
    int n = 0;
    for (int k = k0; k <= k1; ++k)
      if (c->src[k] >= 0 && !seen[c->src[k]]) { seen[c->src[k]] = true; ++n; }
    return n;
  };
  *mode = c->medium_mode;
  const bool planes = c->medium_mode != fdp::M_TABLE;
  *planes_stress = planes ? count(fdp::C_MU, fdp::C_P3) : 0;
  *planes_velocity = planes ? count(fdp::C_EQX, fdp::C_R3W) : 0;
  return FDP_OK;
}

int fdp_core_info(fdp_ctx* c, int32_t* rect8) {
  if (!c || !rect8) return fail(c, FDP_ERR_ARG, "null argument");
  for (int k = 0; k < 4; ++k) {
    rect8[k] = c->use_core ? c->cs[k] : 0;
    rect8[4 + k] = c->use_core ? c->cv[k] : 0;
  }
  return FDP_OK;
}

int fdp_march_info(fdp_ctx* c, int32_t* region8, int32_t* shape4) {
  if (!c || !region8 || !shape4) return fail(c, FDP_ERR_ARG, "null argument");
  const bool on = use_march(c);
  const fdp::MarchGrid& m = c->mg;
  const int32_t r[8] = {m.fx0, m.fx1, m.fz0, m.fz1, m.sx0, m.sx1, m.sz0, m.sz1};
  const int32_t sh[4] = {m.nstrips, c->march_rows, c->march_ctas, c->march_rows};
  for (int k = 0; k < 8; ++k) region8[k] = on ? r[k] : 0;
  for (int k = 0; k < 4; ++k) shape4[k] = on ? sh[k] : 0;
  return FDP_OK;
}

int fdp_get_stream(fdp_ctx* c, void** stream) {
  if (!c || !stream) return fail(c, FDP_ERR_ARG, "null argument");
  *stream = (void*)c->stream;
  return FDP_OK;
}

int fdp_profile_run(fdp_ctx* c, int32_t it_begin, int32_t it_end, double* ms_out, int64_t* launches_out) {
  const TraceRange trace("fdp_profile_run");
  if (!c || !ms_out || !launches_out) return fail(c, FDP_ERR_ARG, "null argument");
  if (!c->have_medium || !c->have_pml || !c->have_nr || !c->have_source)
    return fail(c, FDP_ERR_STATE, "set medium, PML profiles, bottom coefficients and source before profiling");
  if (it_begin < 1 || it_end > c->mt2 || it_end < it_begin)
    return fail(c, FDP_ERR_ARG, "levels %d..%d outside 1..MT2=%d", it_begin, it_end, c->mt2);
  CK(c, cudaSetDevice(c->g.device));
  for (int k = 0; k < 5; ++k) { ms_out[k] = 0.0; launches_out[k] = 0; }
  auto body = [&](auto zero) -> int {
    using T = decltype(zero);
    Params<T> p;
    fill_params<T>(c, p);
    const int nedge = edge_threads(c);
    const bool core[2] = {use_march(c) || (c->use_core && !c->fused[0] && c->cs[1] > c->cs[0]),
                          !use_march(c) && c->use_core && !c->fused[1] && c->cv[1] > c->cv[0]};
    // every level is enqueued before the one synchronisation at the end, so
    // the device never waits for the host and each window holds device time
    // only: per level, events around the two phases and the edge, and
    // around each phase's core kernel
    const int n = it_end - it_begin + 1;
    std::vector<cudaEvent_t> ev((size_t)n * 8, nullptr);
    int rc = FDP_OK;
    for (auto& e : ev)
      if (cudaEventCreate(&e) != cudaSuccess) { e = nullptr; rc = fail(c, FDP_ERR_CUDA, "cudaEventCreate failed"); break; }
    if (rc == FDP_OK) {
      fdp::k_set_base<<<1, 1, 0, c->stream>>>((int*)c->itbase.p, it_begin);
      for (int it = it_begin; it <= it_end && use_march(c); ++it) {
        // march levels: entry 0 the whole level (frames beside the march
        // kernel), entry 2 its k_edge, entry 3 the march kernel
        const int off = it - it_begin;
        cudaEvent_t* e = &ev[(size_t)off * 8];
        c->core_ev[0][0] = e[4];
        c->core_ev[0][1] = e[5];
        cudaEventRecord(e[0], c->stream);
        launch_level_any<T>(c, p, off, true, false);
        cudaEventRecord(e[1], c->stream);
        cudaEventRecord(e[2], c->stream);
        if (nedge > 0) {
          Params<T> pe = p;
          set_fields(c, pe, c->fields, c->fields);
          launch<T>(c, pe, 2, off);
        }
        cudaEventRecord(e[3], c->stream);
      }
      for (int it = it_begin; it <= it_end && !use_march(c); ++it) {
        const int off = it - it_begin;
        cudaEvent_t* e = &ev[(size_t)off * 8];
        for (int k = 0; k < 2; ++k) {
          c->core_ev[k][0] = core[k] ? e[4 + 2 * k] : nullptr;
          c->core_ev[k][1] = core[k] ? e[5 + 2 * k] : nullptr;
        }
        cudaEventRecord(e[0], c->stream);
        launch<T>(c, p, 0, off);
        cudaEventRecord(e[1], c->stream);
        launch<T>(c, p, 1, off);
        cudaEventRecord(e[2], c->stream);
        if (nedge > 0) launch<T>(c, p, 2, off);
        c->launches += fdp::edge_launch(c, off);
        cudaEventRecord(e[3], c->stream);
      }
      fdp::k_add_base<<<1, 1, 0, c->stream>>>((int*)c->itbase.p, n);
      c->launches += 2;
      for (auto& pair : c->core_ev) pair[0] = pair[1] = nullptr;
      cudaError_t err = cudaStreamSynchronize(c->stream);
      if (err == cudaSuccess) err = cudaGetLastError();
      if (err != cudaSuccess) rc = fail(c, FDP_ERR_CUDA, "profile run: %s", cudaGetErrorString(err));
      for (int off = 0; off < n && rc == FDP_OK; ++off) {
        const cudaEvent_t* e = &ev[(size_t)off * 8];
        float t;
        for (int k = 0; k < 3; ++k)
          if (cudaEventElapsedTime(&t, e[k], e[k + 1]) == cudaSuccess) ms_out[k] += t;
        for (int k = 0; k < 2; ++k)
          if (core[k] && cudaEventElapsedTime(&t, e[4 + 2 * k], e[5 + 2 * k]) == cudaSuccess) {
            ms_out[3 + k] += t;
            launches_out[3 + k] += 1;
          }
        launches_out[0] += 1; launches_out[1] += use_march(c) ? 0 : 1; launches_out[2] += nedge > 0 ? 1 : 0;
      }
    }
    for (auto& e : ev) if (e) cudaEventDestroy(e);
    if (rc != FDP_OK) return rc;
    if (it_end > c->last_it) c->last_it = it_end;
    return FDP_OK;
  };
  return c->prec == 8 ? body(0.0) : body(0.0f);
}

const char* fdp_last_error(const fdp_ctx* c) { return c ? c->err.c_str() : g_create_error.c_str(); }

void fdp_destroy(fdp_ctx* c) {
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  fdp::edge_release(c);
  drop_graphs(c);
  unshare_medium(c);
  DevArr* all[] = {&c->jm, &c->coef, &c->planes, &c->aux, &c->ab, &c->hist, &c->stf, &c->rec, &c->raw, &c->itbase,
                   &c->errbuf, &c->frame_s, &c->frame_v, &c->mframe_s, &c->mframe_v, &c->diag_flag};
  for (auto* a : all) if (a->p) cudaFree(a->p);
  for (auto& a : c->fields) if (a.p) cudaFree(a.p);
  for (auto& a : c->alt) if (a.p) cudaFree(a.p);
  for (auto& a : c->prof) if (a.p) cudaFree(a.p);
  for (auto& a : c->mem) if (a.p) cudaFree(a.p);
  if (c->side) cudaStreamSynchronize(c->side);
  if (c->fork) cudaEventDestroy(c->fork);
  if (c->join) cudaEventDestroy(c->join);

  if (c->side) cudaStreamDestroy(c->side);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

}  // extern "C"

// ===========================================================================
// Batched shots (fdp_batch_*): many prepared contexts advanced together.
// Shots are grouped by free-surface mode and medium representation (the
// template parameters of the kernels); each level is one launch per phase
// per group, and runs of kChunk levels are replayed from a CUDA graph.

struct BatchGroup {
  bool si = false;
  int mode = 0;
  int first_shot = 0, n = 0;     // shots [first_shot, first_shot + n) of the sorted order
  int items[5] = {0, 0, 0, 0, 0};     // stress, velocity, edge, stress core, velocity core items
  int resident[5] = {0, 0, 0, 0, 0};  // CTAs of each kernel one SM holds
};

struct fdp_batch {
  std::vector<fdp_ctx*> shots;  // sorted by group
  std::vector<unsigned long long> gens;  // each shot's parameter generation at creation
  std::vector<BatchGroup> groups;
  int prec = 4, device = 0;
  cudaStream_t stream = nullptr;
  DevArr params, first, itbase;  // Params[shots]; per group [5][n+1] first items
  // frame/core split (every shot has one): frame units of all shots, and
  // per group [2][n] offsets of each shot's stress / velocity units
  bool framed = false;
  DevArr units, ubase;
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  int m = 0, waves = 0;          // units per item; persistent CTAs per resident slot (0: one CTA per item)
                                 // m = FDP_BATCH_SHOTS: every shot's own kernels on its own stream
  bool tuned = false;            // shape fixed (by the caller or by tuning)
  int sms = 0;
  cudaGraphExec_t graph = nullptr;
  std::vector<cudaEvent_t> shot_ev;  // per shot: the end of its levels, joined into `stream`
  long long launches = 0;
  std::string err;
};

namespace {

int bfail(fdp_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (b) b->err = buf; else g_create_error = buf;
  return code;
}

#define BCK(b, call)                                                                        \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) return bfail((b), FDP_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// Without the frame/core split the batched unit kernels update every cell.
template <class T> void clear_core(Params<T>& p) {
  p.cs_x0 = p.cs_x1 = p.cs_z0 = p.cs_z1 = 0;
  p.cv_x0 = p.cv_x1 = p.cv_z0 = p.cv_z1 = 0;
}

// first-item offsets of group g inside b->first
size_t group_first_offset(const fdp_batch* b, size_t g) {
  size_t off = 0;
  for (size_t k = 0; k < g; ++k) off += (size_t)5 * (b->groups[k].n + 1);
  return off;
}

// Items of each kernel per shot at m units (core blocks) per item; uploads
// the queues.
int batch_queue(fdp_batch* b) {
  std::vector<int> first;
  for (BatchGroup& G : b->groups) {
    for (int ph = 0; ph < 5; ++ph) {
      int acc = 0;
      for (int s = 0; s < G.n; ++s) {
        const fdp_ctx* c = b->shots[G.first_shot + s];
        first.push_back(acc);
        if (ph < 2 && b->framed) {
          acc += ph == 0 ? c->nframe_s : c->nframe_v;
        } else if (ph < 2) {
          const int rows = fdp::kBZ * (ph == 0 ? fdp::kRZS : fdp::kRZV);
          const int gx = (c->NX + fdp::kBX - 1) / fdp::kBX, gy = (c->NZ + rows - 1) / rows;
          acc += gx * ((gy + b->m - 1) / b->m);
        } else if (ph == 2) {
          acc += (edge_threads(c) + fdp::kBX * fdp::kBZ - 1) / (fdp::kBX * fdp::kBZ);
        } else if (b->framed) {
          const int* r = ph == 3 ? c->cs : c->cv;
          const int gx = ((r[1] - r[0]) / 4 + fdp::kBX - 1) / fdp::kBX, gy = (r[3] - r[2] + fdp::kBZ - 1) / fdp::kBZ;
          acc += (r[1] > r[0]) ? gx * ((gy + b->m - 1) / b->m) : 0;
        }
      }
      first.push_back(acc);
      G.items[ph] = acc;
    }
  }
  cudaError_t e = cudaMemcpyAsync(b->first.p, first.data(), first.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bfail(b, FDP_ERR_CUDA, "batch queue upload: %s", cudaGetErrorString(e));
  return FDP_OK;
}

// Frame units of every shot, copied from the contexts, and their offsets.
int batch_units(fdp_batch* b) {
  size_t total = 0;
  for (const fdp_ctx* c : b->shots) total += (size_t)c->nframe_s + c->nframe_v;
  cudaError_t e = cudaMalloc(&b->units.p, std::max<size_t>(total, 1) * 4 * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&b->ubase.p, std::max<size_t>(2 * b->shots.size(), 1) * sizeof(int));
  if (e != cudaSuccess) return bfail(b, FDP_ERR_ALLOC, "frame unit lists: %s", cudaGetErrorString(e));
  std::vector<int> base(2 * b->shots.size());
  size_t off = 0;
  for (const BatchGroup& G : b->groups)
    for (int ph = 0; ph < 2; ++ph)
      for (int s = 0; s < G.n; ++s) {
        const fdp_ctx* c = b->shots[G.first_shot + s];
        const int n = ph == 0 ? c->nframe_s : c->nframe_v;
        base[2 * G.first_shot + ph * G.n + s] = (int)off;
        e = cudaMemcpyAsync((int*)b->units.p + 4 * off, (ph == 0 ? c->frame_s : c->frame_v).p, (size_t)n * 4 * sizeof(int),
                            cudaMemcpyDeviceToDevice, b->stream);
        if (e != cudaSuccess) return bfail(b, FDP_ERR_CUDA, "frame unit lists: %s", cudaGetErrorString(e));
        off += n;
      }
  e = cudaMemcpyAsync(b->ubase.p, base.data(), base.size() * sizeof(int), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bfail(b, FDP_ERR_CUDA, "frame unit lists: %s", cudaGetErrorString(e));
  return FDP_OK;
}

template <class T, bool SI, int MODE> int group_occupancy(fdp_batch* b, BatchGroup& G) {
  const int threads = fdp::kBX * fdp::kBZ;
  BCK(b, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&G.resident[0], fdp::k_stress_batch<T, SI, MODE>, threads, 0));
  BCK(b, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&G.resident[1], fdp::k_velocity_batch<T, SI, MODE>, threads, 0));
  BCK(b, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&G.resident[2], fdp::k_edge_batch<T, SI>, threads, 0));
  BCK(b, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&G.resident[3], fdp::k_stress_core_batch<T, MODE>, threads, 0));
  BCK(b, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&G.resident[4], fdp::k_velocity_core_batch<T, MODE>, threads, 0));
  return FDP_OK;
}

template <class T> int group_occupancy_any(fdp_batch* b, BatchGroup& G) {
  switch (G.mode) {
    case fdp::M_TABLE: return G.si ? group_occupancy<T, true, fdp::M_TABLE>(b, G) : group_occupancy<T, false, fdp::M_TABLE>(b, G);
    case fdp::M_BIOT: return G.si ? group_occupancy<T, true, fdp::M_BIOT>(b, G) : group_occupancy<T, false, fdp::M_BIOT>(b, G);
    default: return G.si ? group_occupancy<T, true, fdp::M_PLANES>(b, G) : group_occupancy<T, false, fdp::M_PLANES>(b, G);
  }
}

int group_grid(const fdp_batch* b, const BatchGroup& G, int kind) {
  const int items = G.items[kind];
  if (b->waves <= 0) return std::max(items, 1);
  return std::max(1, std::min(items, b->waves * G.resident[kind] * b->sms));
}

template <class T, bool SI, int MODE> void group_level(fdp_batch* b, size_t g, int it_off) {
  const BatchGroup& G = b->groups[g];
  const size_t psize = sizeof(Params<T>);
  const int* ubase = b->ubase.p ? (const int*)b->ubase.p + 2 * G.first_shot : nullptr;
  const fdp::BatchQueue q{(const char*)b->params.p + psize * G.first_shot,
                          (const int*)b->first.p + group_first_offset(b, g), (const int4*)b->units.p, ubase, G.n,
                          b->m, b->framed ? 1 : 0};
  const dim3 blk(fdp::kBX, fdp::kBZ, 1);
  for (int ph = 0; ph < 2; ++ph) {
    const bool core = b->framed && G.items[3 + ph] > 0;
    cudaStream_t fs = core ? b->side : b->stream;
    if (core) {
      cudaEventRecord(b->fork, b->stream);
      cudaStreamWaitEvent(b->side, b->fork, 0);
    }
    if (G.items[ph] > 0) {
      if (ph == 0) fdp::k_stress_batch<T, SI, MODE><<<group_grid(b, G, 0), blk, 0, fs>>>(q, G.items[0], it_off);
      else fdp::k_velocity_batch<T, SI, MODE><<<group_grid(b, G, 1), blk, 0, fs>>>(q, G.items[1], it_off);
      b->launches += 1;
    }
    if (core) {
      if (ph == 0) fdp::k_stress_core_batch<T, MODE><<<group_grid(b, G, 3), blk, 0, b->stream>>>(q, G.items[3]);
      else fdp::k_velocity_core_batch<T, MODE><<<group_grid(b, G, 4), blk, 0, b->stream>>>(q, G.items[4]);
      cudaEventRecord(b->join, b->side);
      cudaStreamWaitEvent(b->stream, b->join, 0);
      b->launches += 1;
    }
  }
  if (G.items[2] > 0) {
    fdp::k_edge_batch<T, SI><<<group_grid(b, G, 2), blk, 0, b->stream>>>(q, G.items[2], it_off);
    b->launches += 1;
  }
}

template <class T> void batch_level(fdp_batch* b, int it_off) {
  for (size_t g = 0; g < b->groups.size(); ++g) {
    const BatchGroup& G = b->groups[g];
    switch (G.mode) {
      case fdp::M_TABLE: G.si ? group_level<T, true, fdp::M_TABLE>(b, g, it_off) : group_level<T, false, fdp::M_TABLE>(b, g, it_off); break;
      case fdp::M_BIOT: G.si ? group_level<T, true, fdp::M_BIOT>(b, g, it_off) : group_level<T, false, fdp::M_BIOT>(b, g, it_off); break;
      default: G.si ? group_level<T, true, fdp::M_PLANES>(b, g, it_off) : group_level<T, false, fdp::M_PLANES>(b, g, it_off);
    }
  }
}

int batch_launches_per_level(const fdp_batch* b) {
  int n = 0;
  for (const BatchGroup& G : b->groups)
    for (int k = 0; k < 5; ++k) n += G.items[k] > 0 && (k < 3 || b->framed) ? 1 : 0;
  return n;
}

// Runs levels [it, it + n) directly (no graph), starting the level counter at it.
template <class T> int batch_direct(fdp_batch* b, int it, int n) {
  fdp::k_set_base<<<1, 1, 0, b->stream>>>((int*)b->itbase.p, it);
  b->launches += 1;
  for (int k = 0; k < n; ++k) batch_level<T>(b, k);
  BCK(b, cudaGetLastError());
  return FDP_OK;
}

int batch_set_shape(fdp_batch* b, int m, int waves) {
  if (b->graph) { cudaGraphExecDestroy(b->graph); b->graph = nullptr; }
  b->m = m;
  b->waves = waves;
  return m == FDP_BATCH_SHOTS ? FDP_OK : batch_queue(b);
}

// Of n levels of the shots mode, those a shot runs as march levels: an
// even number (a march level leaves the other buffers current, and the
// batch's work-queue kernels keep the ones they were given).
int shots_march_levels(fdp_ctx* c, int n) {
  c->batch_march = true;
  const int nm = use_march(c) ? (n & ~1) : 0;
  c->batch_march = false;
  return nm;
}

// The shots mode: n levels of every shot with the shot's own kernels (the
// level sequence fdp_run launches: march levels or the frame/core split,
// folded row-1 and receiver step, one k_edge at the end), each shot on its
// own stream, forked from and joined back to the batch stream.  Shots with
// march levels run one after another (a march kernel's CTAs fill the GPU
// in step with one another; side by side they would contend), the others
// side by side after them.  A shot with march levels runs an even number
// of them as one run and the odd last level, if any, as a run of its own
// in place.  Each shot's level counter starts where the batch set it and
// advances by n at the end.
template <class T> void shots_levels(fdp_batch* b, int n) {
  cudaEventRecord(b->fork, b->stream);
  cudaEvent_t after = b->fork;
  for (int pass = 0; pass < 2; ++pass) {
    const cudaEvent_t start = after;
    for (size_t s = 0; s < b->shots.size(); ++s) {
      fdp_ctx* c = b->shots[s];
      const int nm = shots_march_levels(c, n);
      if ((pass == 0) != (nm > 0)) continue;
      cudaStreamWaitEvent(c->stream, pass == 0 ? after : start, 0);
      Params<T> p;
      if (nm > 0) {
        c->batch_march = true;
        fill_params<T>(c, p);
        for (int k = 0; k < nm; ++k) launch_level_any<T>(c, p, k, k == 0, k == nm - 1);
        c->batch_march = false;
      }
      fill_params<T>(c, p);
      for (int k = nm; k < n; ++k) launch_level_any<T>(c, p, k, k == nm, k == n - 1);
      fdp::k_add_base<<<1, 1, 0, c->stream>>>((int*)c->itbase.p, n);
      cudaEventRecord(b->shot_ev[s], c->stream);
      if (pass == 0) after = b->shot_ev[s];
      else cudaStreamWaitEvent(b->stream, b->shot_ev[s], 0);
    }
  }
  cudaStreamWaitEvent(b->stream, after, 0);
}

long long shots_launches(const fdp_batch* b, int n) {
  long long total = 0;
  for (fdp_ctx* c : b->shots) {
    const int nm = shots_march_levels(c, n);
    if (nm > 0) {
      c->batch_march = true;
      total += run_launches(c, nm);
      c->batch_march = false;
    }
    if (n > nm) total += run_launches(c, n - nm);
    total += 1;
  }
  return total;
}

// Sets every shot's level counter to `it` (on the batch stream).
void shots_set_base(fdp_batch* b, int it) {
  for (fdp_ctx* c : b->shots) fdp::k_set_base<<<1, 1, 0, b->stream>>>((int*)c->itbase.p, it);
  b->launches += (long long)b->shots.size();
}

// The shots mode's graph of kChunk levels of every shot.
template <class T> int shots_graph(fdp_batch* b) {
  if (b->graph) return FDP_OK;
  cudaGraph_t gr = nullptr;
  BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
  std::vector<long long> before;
  for (const fdp_ctx* c : b->shots) before.push_back(c->launches);
  shots_levels<T>(b, kChunk);
  for (size_t s = 0; s < b->shots.size(); ++s) b->shots[s]->launches = before[s];  // capture only records
  cudaError_t e = cudaStreamEndCapture(b->stream, &gr);
  if (e != cudaSuccess) return bfail(b, FDP_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
  e = cudaGraphInstantiate(&b->graph, gr, 0);
  cudaGraphDestroy(gr);
  if (e != cudaSuccess) { b->graph = nullptr; return bfail(b, FDP_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e)); }
  return FDP_OK;
}

// Runs levels [it, it_end] in the shots mode: graph replays of kChunk
// levels, then the rest launched directly.
template <class T> int shots_run(fdp_batch* b, int it, int it_end) {
  shots_set_base(b, it);
  int rc;
  if (it_end - it + 1 >= kChunk && (rc = shots_graph<T>(b)) != FDP_OK) return rc;
  while (it_end - it + 1 >= kChunk) {
    BCK(b, cudaGraphLaunch(b->graph, b->stream));
    b->launches += shots_launches(b, kChunk);
    it += kChunk;
  }
  if (it <= it_end) {
    const long long before = b->launches;
    shots_levels<T>(b, it_end - it + 1);
    b->launches = before + shots_launches(b, it_end - it + 1);
  }
  BCK(b, cudaGetLastError());
  return FDP_OK;
}

// Shape tuning on real levels: every candidate computes the same values bit
// for bit, so the levels spent timing candidates are levels of the run.
// Sets *used to the number of levels run (0 when the run is too short).
template <class T> int batch_tune(fdp_batch* b, int it_begin, int it_end, int* used) {
  static const int kM[] = {1, 2, 4};
  static const int kWaves[] = {0, 1, 2};
  const int per = 2;  // levels per candidate
  *used = 0;
  const int ncand = (int)(sizeof kM / sizeof kM[0]) * (int)(sizeof kWaves / sizeof kWaves[0]);
  if (it_end - it_begin + 1 < ncand * per) return FDP_OK;
  cudaEvent_t e0, e1;
  BCK(b, cudaEventCreate(&e0));
  BCK(b, cudaEventCreate(&e1));
  float best = 1e30f;
  int bm = b->m, bw = b->waves, it = it_begin, rc = FDP_OK;
  for (int m : kM) {
    for (int w : kWaves) {
      if ((rc = batch_set_shape(b, m, w)) != FDP_OK) break;
      cudaEventRecord(e0, b->stream);
      if ((rc = batch_direct<T>(b, it, per)) != FDP_OK) break;
      cudaEventRecord(e1, b->stream);
      float ms = 0.f;
      cudaError_t e = cudaEventSynchronize(e1);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess) { rc = bfail(b, FDP_ERR_CUDA, "shape tuning: %s", cudaGetErrorString(e)); break; }
      if (ms < best) { best = ms; bm = m; bw = w; }
      it += per;
    }
    if (rc != FDP_OK) break;
  }
  // the shots mode, timed over one graph replay of kChunk levels when the
  // run still has them (its direct launches are host-bound)
  if (rc == FDP_OK && it_end - it + 1 >= kChunk) {
    // the graph is built before the clock starts: the device would
    // otherwise wait for its capture and instantiation
    if ((rc = batch_set_shape(b, FDP_BATCH_SHOTS, 0)) == FDP_OK && (rc = shots_graph<T>(b)) == FDP_OK) {
      cudaEventRecord(e0, b->stream);
      rc = shots_run<T>(b, it, it + kChunk - 1);
      cudaEventRecord(e1, b->stream);
      float ms = 0.f;
      cudaError_t e = cudaEventSynchronize(e1);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (rc == FDP_OK && e != cudaSuccess) rc = bfail(b, FDP_ERR_CUDA, "shape tuning: %s", cudaGetErrorString(e));
      if (rc == FDP_OK) {
        if (ms * per / kChunk < best) { best = ms * per / kChunk; bm = FDP_BATCH_SHOTS; bw = 0; }
        it += kChunk;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc != FDP_OK) return rc;
  *used = it - it_begin;
  if (bm == b->m && bw == b->waves) return FDP_OK;  // keeps the shots mode's graph
  return batch_set_shape(b, bm, bw);
}

template <class T> int batch_run_t(fdp_batch* b, int it_begin, int it_end) {
  int it = it_begin;
  if (!b->tuned) {
    int used = 0, rc = batch_tune<T>(b, it_begin, it_end, &used);
    if (rc != FDP_OK) return rc;
    it += used;
    b->tuned = used > 0;
  }
  if (it > it_end) return FDP_OK;
  if (b->m == FDP_BATCH_SHOTS) return shots_run<T>(b, it, it_end);
  fdp::k_set_base<<<1, 1, 0, b->stream>>>((int*)b->itbase.p, it);
  b->launches += 1;
  if (it_end - it + 1 >= kChunk && !b->graph) {
    cudaGraph_t gr = nullptr;
    BCK(b, cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    const long long before = b->launches;
    for (int k = 0; k < kChunk; ++k) batch_level<T>(b, k);
    fdp::k_add_base<<<1, 1, 0, b->stream>>>((int*)b->itbase.p, kChunk);
    b->launches = before;
    cudaError_t e = cudaStreamEndCapture(b->stream, &gr);
    if (e != cudaSuccess) return bfail(b, FDP_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    e = cudaGraphInstantiate(&b->graph, gr, 0);
    cudaGraphDestroy(gr);
    if (e != cudaSuccess) { b->graph = nullptr; return bfail(b, FDP_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(e)); }
  }
  while (it_end - it + 1 >= kChunk && b->graph) {
    BCK(b, cudaGraphLaunch(b->graph, b->stream));
    b->launches += (long long)kChunk * batch_launches_per_level(b) + 1;
    it += kChunk;
  }
  int k = 0;
  for (; it <= it_end; ++it, ++k) batch_level<T>(b, k);
  BCK(b, cudaGetLastError());
  return FDP_OK;
}

}  // namespace

extern "C" {

int fdp_batch_create(fdp_ctx* const* shots, int32_t n, fdp_batch** out) {
  if (!shots || !out || n < 1) return bfail(nullptr, FDP_ERR_ARG, "need at least one shot and an output pointer");
  *out = nullptr;
  for (int s = 0; s < n; ++s) {
    const fdp_ctx* c = shots[s];
    if (!c) return bfail(nullptr, FDP_ERR_ARG, "shot %d is null", s);
    if (!c->have_medium || !c->have_pml || !c->have_nr || !c->have_source)
      return bfail(nullptr, FDP_ERR_STATE, "shot %d: set medium, PML profiles, bottom coefficients and source first", s);
    if (c->mr > 0 && !c->raw.p) return bfail(nullptr, FDP_ERR_STATE, "shot %d: receiver buffer missing", s);
    for (int t = 0; t < s; ++t)
      if (shots[t] == c) return bfail(nullptr, FDP_ERR_ARG, "shot %d appears twice", s);
    if (c->prec != shots[0]->prec || c->g.device != shots[0]->g.device)
      return bfail(nullptr, FDP_ERR_UNSUPPORTED, "shot %d differs from shot 0 in precision or device", s);
  }
  fdp_batch* b = new fdp_batch();
  b->prec = shots[0]->prec;
  b->device = shots[0]->g.device;
  // group by (free-surface mode, medium representation), keeping the order within a group
  for (int si = 0; si < 2; ++si)
    for (int mode : {fdp::M_TABLE, fdp::M_PLANES, fdp::M_BIOT}) {
      BatchGroup G;
      G.si = si != 0;
      G.mode = mode;
      G.first_shot = (int)b->shots.size();
      for (int s = 0; s < n; ++s)
        if ((shots[s]->g.stress_imaging != 0) == G.si && shots[s]->medium_mode == mode) b->shots.push_back(shots[s]);
      G.n = (int)b->shots.size() - G.first_shot;
      if (G.n > 0) b->groups.push_back(G);
    }
  auto bail = [&](int rc) {
    if (!b->err.empty()) g_create_error = b->err;
    fdp_batch_destroy(b);
    return rc;
  };
  int rc;
  cudaError_t e = cudaSetDevice(b->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
  if (e != cudaSuccess) return bail(bfail(b, FDP_ERR_CUDA, "batch stream: %s", cudaGetErrorString(e)));
  for (fdp_ctx* c : b->shots) cudaStreamSynchronize(c->stream);
  // the frame/core split when every shot has it (else the unit kernels over
  // every cell); the frame kernels run on a side stream beside the cores
  b->framed = true;
  for (const fdp_ctx* c : b->shots) b->framed = b->framed && c->use_core;
  e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming);
  b->shot_ev.assign(b->shots.size(), nullptr);
  for (auto& ev : b->shot_ev)
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (e != cudaSuccess) return bail(bfail(b, FDP_ERR_CUDA, "batch events: %s", cudaGetErrorString(e)));
  if (b->framed) {
    e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(bfail(b, FDP_ERR_CUDA, "batch side stream: %s", cudaGetErrorString(e)));
    if ((rc = batch_units(b)) != FDP_OK) return bail(rc);
  }
  const size_t psize = b->prec == 8 ? sizeof(Params<double>) : sizeof(Params<float>);
  auto alloc = [&](DevArr& a, size_t bytes) -> int {
    cudaError_t err = cudaMalloc(&a.p, bytes);
    if (err != cudaSuccess) return bfail(b, FDP_ERR_ALLOC, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(err));
    a.bytes = bytes;
    return FDP_OK;
  };
  if ((rc = alloc(b->params, psize * n)) || (rc = alloc(b->first, sizeof(int) * 5 * (n + b->groups.size()))) ||
      (rc = alloc(b->itbase, sizeof(int))))
    return bail(rc);
  std::vector<unsigned char> host(psize * n);
  for (int s = 0; s < n; ++s) b->gens.push_back(b->shots[s]->gen);
  for (int s = 0; s < n; ++s) {
    if (b->prec == 8) {
      Params<double> p;
      fill_params<double>(b->shots[s], p);
      p.it_base = (const int*)b->itbase.p;
      if (!b->framed) clear_core(p);
      std::memcpy(&host[psize * s], &p, psize);
    } else {
      Params<float> p;
      fill_params<float>(b->shots[s], p);
      p.it_base = (const int*)b->itbase.p;
      if (!b->framed) clear_core(p);
      std::memcpy(&host[psize * s], &p, psize);
    }
  }
  e = cudaMemcpyAsync(b->params.p, host.data(), host.size(), cudaMemcpyHostToDevice, b->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) return bail(bfail(b, FDP_ERR_CUDA, "batch parameters: %s", cudaGetErrorString(e)));
  for (BatchGroup& G : b->groups)
    if ((rc = (b->prec == 8 ? group_occupancy_any<double>(b, G) : group_occupancy_any<float>(b, G))) != FDP_OK)
      return bail(rc);
  if ((rc = batch_set_shape(b, 2, 1)) != FDP_OK) return bail(rc);
  for (fdp_ctx* c : b->shots) c->in_batch = true;  // in-place levels while the batch holds them
  *out = b;
  return FDP_OK;
}

int fdp_batch_set_shape(fdp_batch* b, int32_t units_per_item, int32_t waves) {
  if (!b) return bfail(b, FDP_ERR_ARG, "null batch");
  if (units_per_item == 0) {  // tune again on the next run
    b->tuned = false;
    return FDP_OK;
  }
  if (units_per_item == FDP_BATCH_SHOTS) waves = 0;
  else if (units_per_item < 1 || units_per_item > 64 || waves < 0 || waves > 64)
    return bfail(b, FDP_ERR_ARG, "units per item must be 1..64 (or FDP_BATCH_SHOTS) and waves 0..64");
  BCK(b, cudaSetDevice(b->device));
  BCK(b, cudaStreamSynchronize(b->stream));
  b->tuned = true;
  return batch_set_shape(b, units_per_item, waves);
}

int fdp_batch_get_shape(fdp_batch* b, int32_t* units_per_item, int32_t* waves) {
  if (!b || !units_per_item || !waves) return bfail(b, FDP_ERR_ARG, "null argument");
  *units_per_item = b->m;
  *waves = b->waves;
  return FDP_OK;
}

int fdp_batch_run(fdp_batch* b, int32_t it_begin, int32_t it_end) {
  const TraceRange trace("fdp_batch_run");
  if (!b) return bfail(b, FDP_ERR_ARG, "null batch");
  if (it_end < it_begin) return FDP_OK;
  for (size_t s = 0; s < b->shots.size(); ++s) {
    if (it_begin < 1 || it_end > b->shots[s]->mt2)
      return bfail(b, FDP_ERR_ARG, "levels %d..%d outside 1..MT2=%d of a shot", it_begin, it_end, b->shots[s]->mt2);
    // the batch holds copies of each shot's device parameters
    if (b->shots[s]->gen != b->gens[s])
      return bfail(b, FDP_ERR_STATE, "a shot's medium, source, receivers or edge changed after fdp_batch_create");
  }
  BCK(b, cudaSetDevice(b->device));
  const int rc = b->prec == 8 ? batch_run_t<double>(b, it_begin, it_end) : batch_run_t<float>(b, it_begin, it_end);
  if (rc == FDP_OK)
    for (fdp_ctx* c : b->shots) c->last_it = std::max(c->last_it, (int)it_end);
  return rc;
}

int fdp_batch_synchronize(fdp_batch* b) {
  if (!b) return bfail(b, FDP_ERR_ARG, "null batch");
  BCK(b, cudaStreamSynchronize(b->stream));
  for (fdp_ctx* c : b->shots)
    if (int rc = device_status(c)) return bfail(b, rc, "%s", c->err.c_str());
  return FDP_OK;
}

int64_t fdp_batch_kernel_launches(fdp_batch* b) { return b ? b->launches : 0; }

int fdp_batch_get_stream(fdp_batch* b, void** stream) {
  if (!b || !stream) return bfail(b, FDP_ERR_ARG, "null argument");
  *stream = (void*)b->stream;
  return FDP_OK;
}

const char* fdp_batch_last_error(const fdp_batch* b) { return b ? b->err.c_str() : g_create_error.c_str(); }

void fdp_batch_destroy(fdp_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (fdp_ctx* c : b->shots) c->in_batch = false;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  if (b->side) cudaStreamSynchronize(b->side);
  for (DevArr* a : {&b->params, &b->first, &b->itbase, &b->units, &b->ubase}) if (a->p) cudaFree(a->p);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->join) cudaEventDestroy(b->join);
  for (cudaEvent_t ev : b->shot_ev) if (ev) cudaEventDestroy(ev);
  if (b->side) cudaStreamDestroy(b->side);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

}  // extern "C"
