// Receiver sampling that allocates no device memory (fdp_receivers_noalloc
// in include/fdp.h).
//
// Some hosts cannot call cudaMalloc: a Fortran or C driver whose device
// arrays live in a memory pool it manages itself (a second allocator would
// fragment or overcommit the memory that pool has reserved), or a runtime
// that forbids allocation once it is running (allocation synchronises the
// device and may fail late, in the middle of a survey).  For them this entry
// point takes every input and output as caller-owned device memory and keeps
// its only state -- each receiver's previous sample, which the time
// derivative of STORE_SEISMOGRAMS needs (store_seismograms.F90:65-66,
// 92-93) -- in a fixed static device array instead of allocating one.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>
#include <string>

#include "fdp.h"

namespace {

// Capacity of the static state: the previous u, -w, qx and -qz sample of
// up to FDP_NOALLOC_MAX_RECEIVERS receivers in double precision (512 KiB).
// Every device that loads this library holds the array until exit.
static __device__ __align__(256) unsigned char g_prev_samples[(size_t)FDP_NOALLOC_MAX_RECEIVERS * 4 * sizeof(double)];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
// device address of g_prev_samples per device, and the id of the context it
// was looked up in: a device reset makes a new context, in which the array
// may sit elsewhere, so the address is looked up again there
void* g_prev_ptr[kMaxDevices] = {};
unsigned long long g_prev_ctx[kMaxDevices] = {};

}  // namespace

namespace fdp {
void set_global_error(const char* msg);  // fdp_engine.cu; read back by fdp_last_error(NULL)
}

namespace {

int fail(int code, const char* msg) {
  fdp::set_global_error(msg);
  return code;
}

template <class T>
__global__ void k_receivers_noalloc(const T* um, const T* wm, const T* qx, const T* qz, const T* pres,
                                    const T* txx, int nx, int nz, long long ld, int pmll, const int* rec, int mr,
                                    int flags, T dt, int level, T* out, T* prev) {
  const int j = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (j >= mr) return;
  const int pmlxh = pmll + nx - 1, pmlzh = nz - 1;
  auto at = [&](const T* f, int i, int l) { return f[(long long)l * ld + (i - pmll)]; };
  auto inside = [&](int i, int l) { return i >= pmll && i <= pmlxh && l >= 0 && l <= pmlzh; };
  const int IX = rec[4 * j], LX = rec[4 * j + 1], IZ = rec[4 * j + 2], LZ = rec[4 * j + 3];
  T s[6] = {T(0), T(0), T(0), T(0), T(0), T(0)};
  if (inside(IX, LX)) { s[0] = at(um, IX, LX); s[2] = at(qx, IX, LX); }
  if (inside(IZ, LZ)) { s[1] = -at(wm, IZ, LZ); s[3] = -at(qz, IZ, LZ); }
  if (inside(IZ, LX)) { s[4] = at(pres, IZ, LX); s[5] = -at(txx, IZ, LX); }
  T* p = prev + 4 * (long long)j;
  if (level == 1) {
    // SSU, SSW, SSQX, SSQZ start at zero (alloc_t_seis.F90:70-73)
    p[0] = T(0); p[1] = T(0); p[2] = T(0); p[3] = T(0);
  }
  T* r = out + (long long)j * FDP_REC_VALUES;
#pragma unroll
  for (int k = 0; k < FDP_REC_VALUES; ++k) r[k] = T(0);
  if (flags & FDP_REC_TLV) {
    r[0] = s[0]; r[1] = s[1];
    r[2] = (s[0] - p[0]) / dt; r[3] = (s[1] - p[1]) / dt;
    if (flags & FDP_REC_TLQ) {
      r[4] = s[2]; r[5] = s[3];
      r[6] = (s[2] - p[2]) / dt; r[7] = (s[3] - p[3]) / dt;
    }
  }
  if (flags & FDP_REC_TLP) { r[8] = s[4]; r[9] = s[5]; }
  p[0] = s[0]; p[1] = s[1]; p[2] = s[2]; p[3] = s[3];
}

// Id of the current device's primary context (made current first), through
// the driver entry points the runtime exposes.
int current_context_id(int dev, unsigned long long* id) {
  using GetCurrent = CUresult (*)(CUcontext*);
  using GetId = CUresult (*)(CUcontext, unsigned long long*);
  static GetCurrent get_current = nullptr;
  static GetId get_id = nullptr;
  if (!get_current || !get_id) {
    void* f1 = nullptr;
    void* f2 = nullptr;
    cudaDriverEntryPointQueryResult q1 = cudaDriverEntryPointSymbolNotFound, q2 = q1;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) != cudaSuccess ||
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) != cudaSuccess ||
        q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
      return fail(FDP_ERR_CUDA, "driver entry points cuCtxGetCurrent/cuCtxGetId not found");
    get_current = (GetCurrent)f1;
    get_id = (GetId)f2;
  }
  // cudaSetDevice makes the device's primary context current (creating it
  // when the device has none yet)
  cudaError_t e = cudaSetDevice(dev);
  if (e != cudaSuccess) return fail(FDP_ERR_CUDA, cudaGetErrorString(e));
  CUcontext ctx = nullptr;
  if (get_current(&ctx) != CUDA_SUCCESS || !ctx || get_id(ctx, id) != CUDA_SUCCESS)
    return fail(FDP_ERR_CUDA, "no current CUDA context");
  return FDP_OK;
}

// Device address of the static state on the current device: looked up with
// cudaGetSymbolAddress on the first call on the device, and again only when
// the device's context has changed since (a cudaDeviceReset in between).
int prev_samples_ptr(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(FDP_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(FDP_ERR_ARG, "device ordinal beyond the supported range");
  std::lock_guard<std::mutex> lk(g_mu);
  unsigned long long id = 0;
  int rc = current_context_id(dev, &id);
  if (rc != FDP_OK) return rc;
  if (!g_prev_ptr[dev] || g_prev_ctx[dev] != id) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_prev_samples);
    if (e != cudaSuccess || !p)
      return fail(FDP_ERR_CUDA, (std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());
    g_prev_ptr[dev] = p;
    g_prev_ctx[dev] = id;
  }
  *out = g_prev_ptr[dev];
  return FDP_OK;
}

}  // namespace

extern "C" {

int fdp_receivers_noalloc(int32_t precision, const void* um, const void* wm, const void* qx, const void* qz,
                          const void* pres, const void* txx, int32_t nx, int32_t nz, int32_t ld, int32_t pmll,
                          const int32_t* rec, int32_t mr, int32_t flags, double dt, int32_t level, void* out,
                          void* stream) {
  if (precision != FDP_F32 && precision != FDP_F64) return fail(FDP_ERR_ARG, "precision must be FDP_F32 or FDP_F64");
  if (mr < 0 || mr > FDP_NOALLOC_MAX_RECEIVERS) {
    char buf[160];
    snprintf(buf, sizeof buf, "fdp_receivers_noalloc: %d receivers exceed the static capacity of %d", mr,
             FDP_NOALLOC_MAX_RECEIVERS);
    return fail(FDP_ERR_ARG, buf);
  }
  // the address look-up comes first, so that a call with no receivers sets
  // the device up without launching anything
  void* prev = nullptr;
  int rc = prev_samples_ptr(&prev);
  if (rc != FDP_OK) return rc;
  if (mr == 0) return FDP_OK;
  if (!um || !wm || !qx || !qz || !pres || !txx || !rec || !out) return fail(FDP_ERR_ARG, "null device pointer");
  if (nx < 1 || nz < 1 || ld < nx || level < 1 || !(dt > 0)) return fail(FDP_ERR_ARG, "bad grid, level or DT");
  cudaStream_t s = (cudaStream_t)stream;
  const int threads = 128, blocks = (mr + threads - 1) / threads;
  if (precision == FDP_F64)
    k_receivers_noalloc<double><<<blocks, threads, 0, s>>>(
        (const double*)um, (const double*)wm, (const double*)qx, (const double*)qz, (const double*)pres,
        (const double*)txx, nx, nz, ld, pmll, rec, mr, flags, dt, level, (double*)out, (double*)prev);
  else
    k_receivers_noalloc<float><<<blocks, threads, 0, s>>>(
        (const float*)um, (const float*)wm, (const float*)qx, (const float*)qz, (const float*)pres,
        (const float*)txx, nx, nz, ld, pmll, rec, mr, flags, (float)dt, level, (float*)out, (float*)prev);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(FDP_ERR_CUDA, cudaGetErrorString(e));
  return FDP_OK;
}

}  // extern "C"
