// Private to the library: the context of one shot (include/fdp.h) as the
// engine and the learned-edge code both see it.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>

#include <nvtx3/nvToolsExt.h>

#include "fdp.h"
#include "fdp_core_tma.cuh"
#include "fdp_march.cuh"

struct DevArr {
  void* p = nullptr;
  size_t bytes = 0;
};

// Device arrays of a medium that several contexts use (fdp_share_medium):
// freed when the last context holding the share lets go of it.
struct MediumShare {
  DevArr jm, coef, planes, aux;
  ~MediumShare() {
    for (DevArr* a : {&jm, &coef, &planes, &aux})
      if (a->p) cudaFree(a->p);
  }
};

struct fdp_edge;
struct EdgeState;  // per-context state of an attached learned edge

struct fdp_ctx {
  fdp_grid g{};
  int prec = 4;
  int MX = 0, MZ = 0, TPML = 0, PMLL = 0, PMLXH = 0, PMLZH = 0, NX = 0, NZ = 0, MX1 = 0;
  int pitch = 0, rows_alloc = 0;
  int medium_mode = fdp::M_TABLE;
  int src[fdp::C_NCOEF], neg[fdp::C_NCOEF];
  double cval_d[fdp::C_NCOEF];
  float cval_f[fdp::C_NCOEF];
  int nplanes = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // device memory
  DevArr fields[8];
  DevArr jm, coef, planes, aux, prof[24], mem[27], ab, hist, stf, rec, raw, itbase, errbuf;
  DevArr diag_flag;  // fdp_diag_wait_timeout: a word nothing sets
  // TMA descriptors of the input fields of each phase; use_tma selects the
  // TMA-staged kernels (FDP_KERNEL_VARIANT=tma; the global-load kernels are
  // the default)
  fdp::TmaMaps tma_vel{}, tma_str{};
  bool use_tma = false;
  // frame/core split (the default; FDP_KERNEL_VARIANT=global runs the unit
  // kernels over the whole grid): core rectangles of each phase and the
  // units holding any cell outside them
  bool use_core = false;
  // frame and core of a phase in one launch (else on two streams), per
  // phase: stress, velocity
  bool fused[2] = {false, false};
  // TMA-staged persistent core kernels (FDP_KERNEL_VARIANT=coretma; FP32
  // contexts with a Biot-plane medium): the maps of each phase's 13 copies
  // and the CTAs a launch runs (one per SM)
  bool core_tma_req = false, core_tma = false;
  fdp::CoreMaps cmaps[2]{};
  int core_ctas = 0;
  int cs[4] = {0, 0, 0, 0}, cv[4] = {0, 0, 0, 0};  // x0, x1, z0, z1
  DevArr frame_s, frame_v;
  int nframe_s = 0, nframe_v = 0;
  // the frame kernel of a phase runs on `side`, concurrently with the core
  // kernel on `stream` (fork and join through events, also inside graphs)
  cudaStream_t side = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;

  // fdp_profile_run: events around each phase's core kernel
  cudaEvent_t core_ev[2][2] = {{nullptr, nullptr}, {nullptr, nullptr}};
  int jmnum = 0;
  int mt2 = 0;
  int mr = 0, rec_flags = 0;
  bool have_medium = false, have_pml = false, have_nr = false, have_source = false;
  // set while jm, coef, planes and aux belong to a share with other
  // contexts (the share frees them, not this context)
  std::shared_ptr<MediumShare> medium_share;
  // march levels (the default for FP32 contexts whose levels outgrow L2;
  // FDP_KERNEL_VARIANT=march forces them): each level's interior in one
  // pass, the levels alternating between the two buffers of each wavefield
  // array.  fields[] always holds the current level's buffers and alt[] the
  // other ones; cur tells which of the two allocations fields[] is (0 or 1).
  bool march = false, march_forced = false;  // forced: named by FDP_KERNEL_VARIANT, whatever the grid size
  DevArr alt[8];
  int cur = 0;
  fdp::MarchGrid mg{};
  int march_ctas = 0, march_rows = 8;
  // the frame kernels' rectangles beside the march kernel (stress: F less
  // its band; velocity: F) and their unit lists
  int ms[4] = {0, 0, 0, 0}, mv[4] = {0, 0, 0, 0};
  DevArr mframe_s, mframe_v;
  int nmframe_s = 0, nmframe_v = 0;
  // tensor maps of the march kernel, per current buffer; ready once the
  // medium is set and its launch chosen
  fdp::MarchMaps mmaps[2]{};
  bool march_ready = false;
  // set while a batch holds the context (its kernels update in place);
  // batch_march while the batch's shots mode runs march levels of it, in
  // pairs, so that every batch run ends in the buffers the batch's work-queue
  // kernels were given
  bool in_batch = false, batch_march = false;
  // captured runs of levels, indexed by the current buffer and by their
  // length (1..kRunGraphs); the longest is replayed over and over, a
  // shorter one ends a run
  static constexpr int kRunGraphs = 32;
  cudaGraphExec_t graph[2][kRunGraphs + 1] = {};
  bool params_dirty = true;
  // bumped by every change of the device parameters (set_*, a shared
  // medium, an attached edge); a batch refuses to run a shot whose count
  // moved after fdp_batch_create
  unsigned long long gen = 0;
  long long launches = 0;
  int last_it = 0;  // highest level run so far
  // learned absorbing edge: state (history, tiles) once the context has
  // trained or carried an edge; applied after every level while attached
  EdgeState* edge = nullptr;
  bool edge_attached = false;
};

// An NVTX range around an entry point, for profilers' timelines (nvtx3 is
// header-only: nothing is loaded unless a profiler is attached).
struct TraceRange {
  explicit TraceRange(const char* name) { nvtxRangePushA(name); }
  ~TraceRange() { nvtxRangePop(); }
  TraceRange(const TraceRange&) = delete;
  TraceRange& operator=(const TraceRange&) = delete;
};

// Marks the context's device parameters changed: its captured graph is
// rebuilt before the next run, and batches made earlier refuse to run it.
inline void params_changed(fdp_ctx* c) {
  c->params_dirty = true;
  ++c->gen;
}

namespace fdp {
// Launches the attached learned edge's kernels for level *it_base + it_off
// on the context's stream (none when no edge is attached); returns the
// number of launches.
int edge_launch(fdp_ctx* c, int it_off);
// Frees the context's learned-edge state.
void edge_release(fdp_ctx* c);
}  // namespace fdp
