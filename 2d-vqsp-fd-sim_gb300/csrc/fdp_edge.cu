// Learned absorbing edge (include/fdp_edge.h): the networks, their training
// and their application after each time level.
//
// One CTA of one warp evaluates one tile of up to 32 samples of one network
// ("set" = side x depth), so that a level's samples (about 12 x 520 on a
// 512^2 region) spread over all SMs.  Its inputs are gathered straight from
// the wavefield and the recorded history (or from a host-provided array),
// rounded to bfloat16 into shared memory; the warp runs them through the
// three layers with mma.sync m16n8k16 (bf16 operands, FP32 accumulators
// starting from the bias), tanh on the hidden layers.  Training continues in
// the same CTA, on the tensor cores too: the back-propagated errors of each
// layer (rounded to bf16) times the transposed weights give the previous
// layer's errors, and the errors' transpose times the layer's inputs gives
// each weight gradient, all m16n8k16 products with FP32 accumulation over
// the tile's samples; bias gradients are FP32 sums of the unrounded errors.
// Every operand is staged K-contiguous in shared memory (transposed copies
// where a product contracts over samples).  The CTA writes its tile's
// partial gradient, and a second kernel adds the tiles' partials to the
// gradient in tile order (no atomics: training is bit-reproducible).
// Adam updates FP32 master weights and refreshes their bf16 copies.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fdp.h"
#include "fdp_ctx.h"
#include "fdp_edge.h"

namespace {

using bf16 = __nv_bfloat16;

constexpr int kIn = FDP_EDGE_IN, kHid = FDP_EDGE_HIDDEN, kOut = FDP_EDGE_OUT, kSets = FDP_EDGE_SETS;
constexpr int kDepth = FDP_EDGE_DEPTH;
constexpr int kBand = kDepth + 3;  // columns (rows) of a side's input band
constexpr int oW1 = 0, oB1 = oW1 + kHid * kIn, oW2 = oB1 + kHid, oB2 = oW2 + kHid * kHid, oW3 = oB2 + kHid,
              oB3 = oW3 + kOut * kHid, kSetP = oB3 + kOut;
static_assert(kSetP == FDP_EDGE_SET_PARAMS, "parameter layout of a set");
static_assert(kIn == 3 * 4 * 8, "inputs: 3 levels x 4 cells x 8 fields");
constexpr int kTile = 32;               // samples per CTA (one warp)
constexpr int sX = kIn + 8, sH = kHid + 8;  // padded shared-memory row strides (bf16 elements)
constexpr int sQ = kTile + 8;           // rows of transposed operands: one column per sample
constexpr int sO = 16 + 8;              // output-layer rows padded to one k-step of 16
constexpr int sY = kOut + 1;            // FP32 rows of outputs, errors and strip values

// shared memory of the network kernel (bytes, every array 16-byte aligned)
constexpr size_t al16(size_t b) { return (b + 15) / 16 * 16; }
struct NetSmem {
  // forward: weights, biases, inputs, activations, outputs, targets
  static constexpr size_t W1 = 0, W2 = W1 + al16((size_t)kHid * sX * 2), W3 = W2 + al16((size_t)kHid * sH * 2),
                          B = W3 + al16((size_t)kOut * sH * 2), X = B + al16((size_t)(2 * kHid + kOut) * 4),
                          H1 = X + al16((size_t)kTile * sX * 2), H2 = H1 + al16((size_t)kTile * sH * 2),
                          Y = H2 + al16((size_t)kTile * sH * 2), Tg = Y + al16((size_t)kTile * kOut * 4),
                          infer = Tg + al16((size_t)kTile * kOut * 4);
  // training: transposed weights and activations, errors
  static constexpr size_t W2T = infer, W3T = W2T + al16((size_t)kHid * sH * 2), XT = W3T + al16((size_t)kHid * sO * 2),
                          H1T = XT + al16((size_t)kIn * sQ * 2), H2T = H1T + al16((size_t)kHid * sQ * 2),
                          V = H2T + al16((size_t)kHid * sQ * 2), DY = V + al16((size_t)kTile * sY * 4),
                          DYb = DY + al16((size_t)kTile * sY * 4), DYT = DYb + al16((size_t)kTile * sO * 2),
                          D2 = DYT + al16((size_t)16 * sQ * 2), D2T = D2 + al16((size_t)kTile * sH * 2),
                          D1T = D2T + al16((size_t)kHid * sQ * 2), train = D1T + al16((size_t)kHid * sQ * 2);
};
constexpr size_t kSmInfer = NetSmem::infer;
constexpr size_t kSmTrain = NetSmem::train;
// Damping output: a strip value v becomes v * (1 - alpha), alpha =
// sigmoid(y + kDampBias) per field, so a new network (y = 0) damps by 1.8 %.
constexpr float kDampBias = -4.f;

// Wavefield view of one FP32 context: pointers at (PMLL, 0).
struct View {
  float* f[8];
  int pitch, PMLL, PMLXH, PMLZH, NX, NZ;
};

// Where a sample lives: set = side * kDepth + depth; sample i of the set.
struct Geometry {
  int PMLL, PMLXH, PMLZH, NX, NZ;
  int Rf;  // floats of one field of one history slot
  __device__ __forceinline__ void cell(int set, int i, int k, int& I, int& L) const {
    const int side = set / kDepth, depth = set % kDepth;
    if (side == 0) { I = PMLL + depth + k; L = i; }
    else if (side == 1) { I = PMLXH - depth - k; L = i; }
    else { I = PMLL + kDepth + i; L = PMLZH - depth - k; }
  }
  // history index of band cell (side, depth c, i) within one field of a slot
  __device__ __forceinline__ int hidx(int side, int c, int i) const {
    if (side == 0) return i * kBand + c;
    if (side == 1) return NZ * kBand + i * kBand + c;
    return 2 * NZ * kBand + c * NX + (kDepth + i);
  }
};

__host__ __device__ inline int set_count(int set, int NX, int NZ) {
  return set / kDepth < 2 ? NZ : NX - 2 * kDepth;
}

__device__ __forceinline__ int slot_of(int level) { return ((level % 3) + 3) % 3; }

struct NetArgs {
  const bf16* wb;      // bf16 weights, kSets * kSetP (biases unused)
  const float* wf;     // FP32 master parameters (biases read from here)
  const float* scale;  // [8]
  const int4* tiles;   // (set, first, count, out_base)
  float* grad;         // training: gradient accumulator, kSets * kSetP
  double* loss;        // training: sum of squared errors
  float* part;         // training: each tile's gradient of its set, [tiles][kSetP]
  double* tloss;       // training: each tile's sum of squared errors
  float gscale;        // training: d loss / d y factor, 2 / (outputs in the batch)
  int damping;         // band source: outputs are damping factors, not corrections
  // array source
  const float* x;      // [.][kIn]
  const float* target;  // [.][kOut]
  float* y;            // [.][kOut]
  // band source
  View t;              // the context the edge corrects
  const float* hist;   // [3][8][Rf] history (post-correction or target values)
  Geometry geo;
  const int* it_base;  // level = (it_base ? *it_base : 0) + it_off
  int it_off;
  View e;              // training: the target context
  int ox;              // target column of the context's column I is I + ox
};

__device__ __forceinline__ uint32_t ld32(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One layer for the warp's 32 rows r0..r0+31: z = bias + in . W^T (in: bf16
// [rows][K] stride si; W: bf16 [N][K] stride sw).  Hidden layers store
// bf16(tanh(z)) into hb (stride sh); the output layer stores z into yf.
template <int K, int N, bool HIDDEN>
__device__ __forceinline__ void warp_layer(const bf16* in, int si, const bf16* W, int sw, const float* bias, int r0,
                                           bf16* hb, int sh, float* yf) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
    const int rb = r0 + 16 * mt;
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) {
      const int n0 = nt * 8;
      float d[4] = {bias[n0 + 2 * t], bias[n0 + 2 * t + 1], bias[n0 + 2 * t], bias[n0 + 2 * t + 1]};
#pragma unroll
      for (int ks = 0; ks < K / 16; ++ks) {
        const int k0 = ks * 16 + 2 * t;
        const uint32_t a[4] = {ld32(in + (rb + g) * si + k0), ld32(in + (rb + g + 8) * si + k0),
                               ld32(in + (rb + g) * si + k0 + 8), ld32(in + (rb + g + 8) * si + k0 + 8)};
        mma_bf16(d, a, ld32(W + (n0 + g) * sw + k0), ld32(W + (n0 + g) * sw + k0 + 8));
      }
      if (HIDDEN) {
        hb[(rb + g) * sh + n0 + 2 * t] = __float2bfloat16_rn(tanhf(d[0]));
        hb[(rb + g) * sh + n0 + 2 * t + 1] = __float2bfloat16_rn(tanhf(d[1]));
        hb[(rb + g + 8) * sh + n0 + 2 * t] = __float2bfloat16_rn(tanhf(d[2]));
        hb[(rb + g + 8) * sh + n0 + 2 * t + 1] = __float2bfloat16_rn(tanhf(d[3]));
      } else {
        yf[(rb + g) * kOut + n0 + 2 * t] = d[0];
        yf[(rb + g) * kOut + n0 + 2 * t + 1] = d[1];
        yf[(rb + g + 8) * kOut + n0 + 2 * t] = d[2];
        yf[(rb + g + 8) * kOut + n0 + 2 * t + 1] = d[3];
      }
    }
  }
}

enum Src { SRC_ARRAY = 0, SRC_BAND = 1 };

// One 16 x 8 tile of D = A . B^T on the tensor cores: A [16 rows][K] and
// B^T [8 rows][K], both bf16 with K contiguous (strides sa, sb elements),
// K a multiple of 16; d the FP32 accumulators (rows g and g+8, columns 2t
// and 2t+1 of the tile, g = lane / 4, t = lane % 4).
template <int K>
__device__ __forceinline__ void mma_tile(float (&d)[4], const bf16* A, int sa, const bf16* B, int sb) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int ks = 0; ks < K / 16; ++ks) {
    const int k0 = ks * 16 + 2 * t;
    const uint32_t a[4] = {ld32(A + g * sa + k0), ld32(A + (g + 8) * sa + k0), ld32(A + g * sa + k0 + 8),
                           ld32(A + (g + 8) * sa + k0 + 8)};
    mma_bf16(d, a, ld32(B + g * sb + k0), ld32(B + g * sb + k0 + 8));
  }
}

// Sum over the 32 samples of a 32 x 8 block of FP32 errors held as two
// m16n8 accumulator tiles (e[mt][4]): per column 2t and 2t+1, the sum of
// the lane's four rows, then over the eight lanes sharing t (a fixed
// shuffle tree: the same order every time).
__device__ __forceinline__ float2 column_sums(const float (&e)[2][4]) {
  float s0 = (e[0][0] + e[0][2]) + (e[1][0] + e[1][2]);
  float s1 = (e[0][1] + e[0][3]) + (e[1][1] + e[1][3]);
#pragma unroll
  for (int off = 4; off < 32; off <<= 1) {
    s0 += __shfl_xor_sync(0xffffffffu, s0, off);
    s1 += __shfl_xor_sync(0xffffffffu, s1, off);
  }
  return make_float2(s0, s1);
}

// One tile of samples through the network; TRAIN adds the backward pass.
// Output: array source -> y[first + s]; band source -> y[out_base + s] (the
// correction buffer).  Inputs of a band sample: 3 levels (new, the history
// of the previous two) x 4 cells inward from the strip cell x 8 fields,
// each divided by the field's scale; its target (training) is the target
// context's value minus the context's value at the strip cell, scaled.
template <int SRC, bool TRAIN>
__global__ void __launch_bounds__(kTile) k_net(const __grid_constant__ NetArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  using M = NetSmem;
  bf16* W1 = reinterpret_cast<bf16*>(smem + M::W1);
  bf16* W2 = reinterpret_cast<bf16*>(smem + M::W2);
  bf16* W3 = reinterpret_cast<bf16*>(smem + M::W3);
  float* B1 = reinterpret_cast<float*>(smem + M::B);
  float* B2 = B1 + kHid;
  float* B3 = B2 + kHid;
  bf16* X = reinterpret_cast<bf16*>(smem + M::X);
  bf16* H1 = reinterpret_cast<bf16*>(smem + M::H1);
  bf16* H2 = reinterpret_cast<bf16*>(smem + M::H2);
  float* Y = reinterpret_cast<float*>(smem + M::Y);
  float* Tg = reinterpret_cast<float*>(smem + M::Tg);
  float* V = reinterpret_cast<float*>(smem + M::V);  // training only
  const int4 tile = a.tiles[blockIdx.x];
  const int set = tile.x, first = tile.y, count = tile.z;
  const int tid = threadIdx.x;
  // weights of the set, 8 bf16 per 16-byte load (every matrix and row of
  // the set starts on a 16-byte boundary: kSetP, oW2, oW3, kIn and kHid are
  // multiples of 8, as are the shared-memory strides)
  static_assert(kSetP % 8 == 0 && oW2 % 8 == 0 && oW3 % 8 == 0 && kIn % 8 == 0 && kHid % 8 == 0 && sX % 8 == 0 &&
                    sH % 8 == 0, "16-byte weight loads");
  const bf16* wb = a.wb + (size_t)set * kSetP;
  const float* wf = a.wf + (size_t)set * kSetP;
  {
    constexpr int n1 = kHid * kIn / 8, n2 = kHid * kHid / 8, n3 = kOut * kHid / 8;
    uint4 v1[n1 / kTile], v2[n2 / kTile], v3[n3 / kTile];
#pragma unroll
    for (int r = 0; r < n1 / kTile; ++r) v1[r] = reinterpret_cast<const uint4*>(wb + oW1)[tid + r * kTile];
#pragma unroll
    for (int r = 0; r < n2 / kTile; ++r) v2[r] = reinterpret_cast<const uint4*>(wb + oW2)[tid + r * kTile];
#pragma unroll
    for (int r = 0; r < n3 / kTile; ++r) v3[r] = reinterpret_cast<const uint4*>(wb + oW3)[tid + r * kTile];
#pragma unroll
    for (int r = 0; r < n1 / kTile; ++r) {
      const int k = 8 * (tid + r * kTile);
      *reinterpret_cast<uint4*>(W1 + (k / kIn) * sX + k % kIn) = v1[r];
    }
#pragma unroll
    for (int r = 0; r < n2 / kTile; ++r) {
      const int k = 8 * (tid + r * kTile);
      *reinterpret_cast<uint4*>(W2 + (k / kHid) * sH + k % kHid) = v2[r];
    }
#pragma unroll
    for (int r = 0; r < n3 / kTile; ++r) {
      const int k = 8 * (tid + r * kTile);
      *reinterpret_cast<uint4*>(W3 + (k / kHid) * sH + k % kHid) = v3[r];
    }
    static_assert(n1 % kTile == 0 && n2 % kTile == 0 && n3 % kTile == 0, "weight loads per lane");
  }
  for (int k = tid; k < kHid; k += kTile) { B1[k] = wf[oB1 + k]; B2[k] = wf[oB2 + k]; }
  if (tid < kOut) B3[tid] = wf[oB3 + tid];
  // inputs (and targets) of sample tid
  const bool valid = tid < count;
  const int i = first + tid;
  float scl[8];
#pragma unroll
  for (int f = 0; f < 8; ++f) scl[f] = a.scale[f];
  if (SRC == SRC_ARRAY) {
    for (int k = 0; k < kIn; ++k) X[tid * sX + k] = __float2bfloat16_rn(valid ? a.x[(size_t)i * kIn + k] : 0.f);
    if (TRAIN)
      for (int o = 0; o < kOut; ++o) Tg[tid * kOut + o] = valid ? a.target[(size_t)i * kOut + o] : 0.f;
  } else {
    const int level = (a.it_base ? *a.it_base : 0) + a.it_off;
    const int side = set / kDepth, depth = set % kDepth;
    const float* h1 = a.hist + (size_t)slot_of(level - 1) * 8 * a.geo.Rf;
    const float* h2 = a.hist + (size_t)slot_of(level - 2) * 8 * a.geo.Rf;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      int I = 0, L = 0;
      if (valid) a.geo.cell(set, i, k, I, L);
      const long long c = (long long)L * a.t.pitch + (I - a.t.PMLL);
      const int hi = valid ? a.geo.hidx(side, depth + k, i) : 0;
#pragma unroll
      for (int f = 0; f < 8; ++f) {
        const float v0 = valid ? a.t.f[f][c] : 0.f;
        const float v1 = valid ? h1[(size_t)f * a.geo.Rf + hi] : 0.f;
        const float v2 = valid ? h2[(size_t)f * a.geo.Rf + hi] : 0.f;
        X[tid * sX + (0 * 4 + k) * 8 + f] = __float2bfloat16_rn(v0 / scl[f]);
        X[tid * sX + (1 * 4 + k) * 8 + f] = __float2bfloat16_rn(v1 / scl[f]);
        X[tid * sX + (2 * 4 + k) * 8 + f] = __float2bfloat16_rn(v2 / scl[f]);
      }
    }
    if (TRAIN) {
      int I = 0, L = 0;
      if (valid) a.geo.cell(set, i, 0, I, L);
      const long long c = (long long)L * a.t.pitch + (I - a.t.PMLL);
      const long long ce = (long long)L * a.e.pitch + (I + a.ox - a.e.PMLL);
#pragma unroll
      for (int f = 0; f < 8; ++f) {
        const float v = valid ? a.t.f[f][c] : 0.f;
        Tg[tid * kOut + f] = valid ? (a.e.f[f][ce] - v) / scl[f] : 0.f;
        V[tid * sY + f] = v / scl[f];
      }
    }
  }
  __syncwarp();
  // forward
  warp_layer<kIn, kHid, true>(X, sX, W1, sX, B1, 0, H1, sH, nullptr);
  __syncwarp();
  warp_layer<kHid, kHid, true>(H1, sH, W2, sH, B2, 0, H2, sH, nullptr);
  __syncwarp();
  warp_layer<kHid, kOut, false>(H2, sH, W3, sH, B3, 0, nullptr, 0, Y);
  __syncwarp();
  if (valid && a.y) {
    float* out = a.y + (size_t)(SRC == SRC_ARRAY ? i : tile.w + tid) * kOut;
#pragma unroll
    for (int o = 0; o < kOut; ++o) out[o] = Y[tid * kOut + o];
  }
  if constexpr (TRAIN) {
    bf16* W2T = reinterpret_cast<bf16*>(smem + M::W2T);
    bf16* W3T = reinterpret_cast<bf16*>(smem + M::W3T);
    bf16* XT = reinterpret_cast<bf16*>(smem + M::XT);
    bf16* H1T = reinterpret_cast<bf16*>(smem + M::H1T);
    bf16* H2T = reinterpret_cast<bf16*>(smem + M::H2T);
    float* DY = reinterpret_cast<float*>(smem + M::DY);
    bf16* DYb = reinterpret_cast<bf16*>(smem + M::DYb);
    bf16* DYT = reinterpret_cast<bf16*>(smem + M::DYT);
    bf16* D2 = reinterpret_cast<bf16*>(smem + M::D2);
    bf16* D2T = reinterpret_cast<bf16*>(smem + M::D2T);
    bf16* D1T = reinterpret_cast<bf16*>(smem + M::D1T);
    const bf16 zero = __float2bfloat16_rn(0.f);
    // transposed operands: weights W2^T, W3^T (output rows padded to 16),
    // and the sample's column of X^T, H1^T, H2^T
    for (int k = tid; k < kHid * kHid; k += kTile) W2T[(k % kHid) * sH + k / kHid] = W2[(k / kHid) * sH + k % kHid];
    for (int k = tid; k < kHid * 16; k += kTile) {
      const int j = k / 16, o = k % 16;
      W3T[j * sO + o] = o < kOut ? W3[o * sH + j] : zero;
    }
    for (int k = 0; k < kIn; ++k) XT[k * sQ + tid] = X[tid * sX + k];
    for (int k = 0; k < kHid; ++k) {
      H1T[k * sQ + tid] = H1[tid * sH + k];
      H2T[k * sQ + tid] = H2[tid * sH + k];
    }
    // output error of sample tid: d loss / d y
    float se = 0.f;
#pragma unroll
    for (int o = 0; o < kOut; ++o) {
      const float y = Y[tid * kOut + o];
      float dy;
      if (SRC == SRC_BAND && a.damping) {
        // prediction -alpha * v of the scaled correction
        const float al = 1.f / (1.f + expf(-(y + kDampBias)));
        const float v = V[tid * sY + o];
        const float r = valid ? -al * v - Tg[tid * kOut + o] : 0.f;
        se += r * r;
        dy = r * a.gscale * (-v) * al * (1.f - al);
      } else {
        const float r = valid ? y - Tg[tid * kOut + o] : 0.f;
        se += r * r;
        dy = r * a.gscale;
      }
      DY[tid * sY + o] = dy;
      const bf16 b = __float2bfloat16_rn(dy);
      DYb[tid * sO + o] = b;
      DYb[tid * sO + kOut + o] = zero;
      DYT[o * sQ + tid] = b;
      DYT[(kOut + o) * sQ + tid] = zero;
    }
    // sum of squared errors of the tile (a fixed shuffle tree); the
    // partials of all tiles are added in tile order by k_grad_reduce, so a
    // training step is bit-reproducible
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) se += __shfl_xor_sync(0xffffffffu, se, off);
    if (tid == 0) a.tloss[blockIdx.x] = (double)se;
    __syncwarp();
    float* grad = a.part + (size_t)blockIdx.x * kSetP;
    const int g = tid >> 2, t = tid & 3;
    // hidden layer 2: E2 = (dY . W3) * (1 - H2^2); bf16 copies E2 (rows) and
    // E2^T; bias gradient from the FP32 values
    for (int nt = 0; nt < kHid / 8; ++nt) {
      float e[2][4];
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        mma_tile<16>(d, DYb + 16 * mt * sO, sO, W3T + 8 * nt * sO, sO);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int q = 16 * mt + g + 8 * (r >> 1), j = 8 * nt + 2 * t + (r & 1);
          const float h = __bfloat162float(H2[q * sH + j]);
          e[mt][r] = d[r] * (1.f - h * h);
          const bf16 b = __float2bfloat16_rn(e[mt][r]);
          D2[q * sH + j] = b;
          D2T[j * sQ + q] = b;
        }
      }
      const float2 sum = column_sums(e);
      if (g == 0) { grad[oB2 + 8 * nt + 2 * t] = sum.x; grad[oB2 + 8 * nt + 2 * t + 1] = sum.y; }
    }
    __syncwarp();
    // hidden layer 1: E1 = (E2 . W2) * (1 - H1^2); bf16 E1^T
    for (int nt = 0; nt < kHid / 8; ++nt) {
      float e[2][4];
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        mma_tile<kHid>(d, D2 + 16 * mt * sH, sH, W2T + 8 * nt * sH, sH);
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          const int q = 16 * mt + g + 8 * (r >> 1), k = 8 * nt + 2 * t + (r & 1);
          const float h = __bfloat162float(H1[q * sH + k]);
          e[mt][r] = d[r] * (1.f - h * h);
          D1T[k * sQ + q] = __float2bfloat16_rn(e[mt][r]);
        }
      }
      const float2 sum = column_sums(e);
      if (g == 0) { grad[oB1 + 8 * nt + 2 * t] = sum.x; grad[oB1 + 8 * nt + 2 * t + 1] = sum.y; }
    }
    __syncwarp();
    // weight gradients over the tile's samples: dW3 = dY^T . H2 (rows 8..15
    // of the padded dY^T are zero), dW2 = E2^T . H1, dW1 = E1^T . X
    for (int nt = 0; nt < kHid / 8; ++nt) {
      float d[4] = {0.f, 0.f, 0.f, 0.f};
      mma_tile<kTile>(d, DYT, sQ, H2T + 8 * nt * sQ, sQ);
      grad[oW3 + g * kHid + 8 * nt + 2 * t] = d[0];
      grad[oW3 + g * kHid + 8 * nt + 2 * t + 1] = d[1];
    }
    for (int mt = 0; mt < kHid / 16; ++mt)
      for (int nt = 0; nt < kHid / 8; ++nt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        mma_tile<kTile>(d, D2T + 16 * mt * sQ, sQ, H1T + 8 * nt * sQ, sQ);
        const int j = 16 * mt + g, k = 8 * nt + 2 * t;
        grad[oW2 + j * kHid + k] = d[0];
        grad[oW2 + j * kHid + k + 1] = d[1];
        grad[oW2 + (j + 8) * kHid + k] = d[2];
        grad[oW2 + (j + 8) * kHid + k + 1] = d[3];
      }
    for (int mt = 0; mt < kHid / 16; ++mt)
      for (int nt = 0; nt < kIn / 8; ++nt) {
        float d[4] = {0.f, 0.f, 0.f, 0.f};
        mma_tile<kTile>(d, D1T + 16 * mt * sQ, sQ, XT + 8 * nt * sQ, sQ);
        const int k = 16 * mt + g, c = 8 * nt + 2 * t;
        grad[oW1 + k * kIn + c] = d[0];
        grad[oW1 + k * kIn + c + 1] = d[1];
        grad[oW1 + (k + 8) * kIn + c] = d[2];
        grad[oW1 + (k + 8) * kIn + c + 1] = d[3];
      }
    // output-layer bias: the FP32 output errors summed over samples in order
    if (tid < kOut) {
      float s = 0.f;
      for (int q = 0; q < kTile; ++q) s += DY[q * sY + tid];
      grad[oB3 + tid] = s;
    }
  }
}

// Adds the tiles' partial gradients to the gradient of their sets, each
// parameter's partials in tile order, and their losses to the loss.  The
// tiles are sorted by set, so a set's tiles are the range a binary search
// finds.
__global__ void k_grad_reduce(const int4* __restrict__ tiles, int ntiles, const float* __restrict__ part,
                              const double* __restrict__ tloss, float* grad, double* loss) {
  const int k = (int)(blockIdx.x * blockDim.x + threadIdx.x);
  if (k == 0) {
    double t = *loss;
    for (int q = 0; q < ntiles; ++q) t += tloss[q];
    *loss = t;
  }
  if (k >= kSets * kSetP) return;
  const int set = k / kSetP, e = k % kSetP;
  // the set's tiles [first, end): known up front, so the loads of the
  // partials go out ahead of the additions, which stay in tile order
  auto bound = [&](int s) {  // first tile of a set >= s
    int lo = 0, hi = ntiles;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (tiles[mid].x < s) lo = mid + 1; else hi = mid;
    }
    return lo;
  };
  const int first = bound(set), end = bound(set + 1);
  float g = grad[k];
#pragma unroll 8
  for (int q = first; q < end; ++q) g += part[(size_t)q * kSetP + e];
  grad[k] = g;
}

// Adam on every parameter; zeroes the gradient and refreshes the bf16 copy.
__global__ void k_adam(float* w, bf16* wb, float* m, float* v, float* g, int n, float lr, float c1, float c2) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const float gk = g[k];
  const float mk = 0.9f * m[k] + 0.1f * gk;
  const float vk = 0.999f * v[k] + 0.001f * gk * gk;
  m[k] = mk;
  v[k] = vk;
  const float mh = mk / c1, vh = vk / c2;
  const float wk = w[k] - lr * mh / (sqrtf(vh) + 1e-8f);
  w[k] = wk;
  wb[k] = __float2bfloat16_rn(wk);
  g[k] = 0.f;
}

__global__ void k_to_bf16(const float* w, bf16* wb, int n) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) wb[k] = __float2bfloat16_rn(w[k]);
}

// Writes the band values of level `level` into their history slot; strip
// cells (depth < kDepth) first receive their correction.  One thread per
// band cell: side blockIdx.z, depth c0 + blockIdx.y, index i along the side.
// Launched for the strip depths, then for the others: a left or right band
// cell beyond the strip can be a bottom strip cell, whose history must be
// its corrected value.
__global__ void k_edge_commit(View t, Geometry geo, float* hist, const float* corr, const int* set_out_base,
                              const float* scale, const int* it_base, int it_off, int c0, int damping) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c = c0 + blockIdx.y, side = blockIdx.z;
  const int count = side < 2 ? geo.NZ : geo.NX - 2 * kDepth;
  if (i >= count) return;
  const int level = (it_base ? *it_base : 0) + it_off;
  int I, L;
  geo.cell(side * kDepth, i, c, I, L);  // depth 0, k = c: the band cell at depth c
  const long long cell = (long long)L * t.pitch + (I - t.PMLL);
  float* h = hist + (size_t)slot_of(level) * 8 * geo.Rf + geo.hidx(side, c, i);
  const float* cr = (corr && c < kDepth) ? corr + (size_t)(set_out_base[side * kDepth + c] + i) * kOut : nullptr;
#pragma unroll
  for (int f = 0; f < 8; ++f) {
    float v = t.f[f][cell];
    if (cr) {
      v = damping ? v * (1.f - 1.f / (1.f + expf(-(cr[f] + kDampBias)))) : v + cr[f] * scale[f];
      t.f[f][cell] = v;
    }
    h[(size_t)f * geo.Rf] = v;
  }
}

// Teacher forcing: the context's whole grid takes the target's values, and
// its band the target's values as history of level `level`.
__global__ void k_edge_teacher(View t, View e, int ox, Geometry geo, float* hist, int level) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int L = blockIdx.y;
  if (x >= t.NX) return;
  const int I = t.PMLL + x;
  const long long ct = (long long)L * t.pitch + x;
  const long long ce = (long long)L * e.pitch + (I + ox - e.PMLL);
  float v[8];
#pragma unroll
  for (int f = 0; f < 8; ++f) {
    v[f] = e.f[f][ce];
    t.f[f][ct] = v[f];
  }
  float* h = hist + (size_t)slot_of(level) * 8 * geo.Rf;
  auto put = [&](int idx) {
#pragma unroll
    for (int f = 0; f < 8; ++f) h[(size_t)f * geo.Rf + idx] = v[f];
  };
  if (I - t.PMLL < kBand) put(geo.hidx(0, I - t.PMLL, L));
  if (t.PMLXH - I < kBand) put(geo.hidx(1, t.PMLXH - I, L));
  if (t.PMLZH - L < kBand && I >= t.PMLL + kDepth && I <= t.PMLXH - kDepth)
    put(geo.hidx(2, t.PMLZH - L, I - t.PMLL - kDepth));
}

}  // namespace

// ---------------------------------------------------------------------------
// host side

struct fdp_edge {
  int device = 0;
  cudaStream_t stream = nullptr;
  DevArr w, wb, m, v, g, scale, loss;
  DevArr part, tloss;         // training: per-tile partial gradients and losses
  DevArr ax, at, ay, atiles;  // array-source scratch
  float hscale[8] = {1, 1, 1, 1, 1, 1, 1, 1};
  int damping = 0;  // band outputs: damping factors instead of corrections
  long long step = 0;
  std::string err;
};

struct EdgeState {
  fdp_edge* net = nullptr;  // applied after every level when set
  Geometry geo{};
  DevArr tiles, set_base, hist, corr;
  int ntiles = 0, nsamples = 0;
};

namespace {

std::string g_edge_error;

int efail(fdp_edge* e, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  if (e) e->err = buf; else g_edge_error = buf;
  return code;
}

#define ECK(e, call)                                                                        \
  do {                                                                                      \
    cudaError_t e_ = (call);                                                                \
    if (e_ != cudaSuccess) return efail((e), FDP_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

int ealloc(fdp_edge* e, DevArr& a, size_t bytes) {
  if (a.p && a.bytes >= bytes) return FDP_OK;
  if (a.p) { cudaFree(a.p); a.p = nullptr; a.bytes = 0; }
  if (bytes == 0) return FDP_OK;
  ECK(e, cudaMalloc(&a.p, bytes));
  a.bytes = bytes;
  return FDP_OK;
}

constexpr size_t kAll = (size_t)kSets * kSetP;

int sync_scale(fdp_edge* e) {
  ECK(e, cudaMemcpyAsync(e->scale.p, e->hscale, sizeof e->hscale, cudaMemcpyHostToDevice, e->stream));
  ECK(e, cudaStreamSynchronize(e->stream));
  return FDP_OK;
}

int refresh_bf16(fdp_edge* e) {
  k_to_bf16<<<(unsigned)((kAll + 255) / 256), 256, 0, e->stream>>>((const float*)e->w.p, (bf16*)e->wb.p, (int)kAll);
  ECK(e, cudaGetLastError());
  return FDP_OK;
}

View view_of(fdp_ctx* c) {
  View v{};
  const size_t off = (size_t)fdp::kPadZ * c->pitch + fdp::kPadX;
  for (int f = 0; f < 8; ++f) v.f[f] = (float*)c->fields[f].p + off;
  v.pitch = c->pitch; v.PMLL = c->PMLL; v.PMLXH = c->PMLXH; v.PMLZH = c->PMLZH; v.NX = c->NX; v.NZ = c->NZ;
  return v;
}

int set_smem_limits(fdp_edge* e) {
  static bool done[64] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev >= 0 && dev < 64 && done[dev]) return FDP_OK;
  ECK(e, cudaFuncSetAttribute(k_net<SRC_ARRAY, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmInfer));
  ECK(e, cudaFuncSetAttribute(k_net<SRC_BAND, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmInfer));
  ECK(e, cudaFuncSetAttribute(k_net<SRC_ARRAY, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmTrain));
  ECK(e, cudaFuncSetAttribute(k_net<SRC_BAND, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmTrain));
  if (dev >= 0 && dev < 64) done[dev] = true;
  return FDP_OK;
}

// Per-context state: tiles of every set, history, correction buffer.
int edge_state(fdp_edge* e, fdp_ctx* c, EdgeState** res) {
  if (c->edge) { *res = c->edge; return FDP_OK; }
  if (c->prec != 4) return efail(e, FDP_ERR_UNSUPPORTED, "the learned edge runs on FP32 contexts");
  if (c->NX < 2 * kBand + 1 || c->NZ < kBand + 1) return efail(e, FDP_ERR_ARG, "grid too small for the edge");
  EdgeState* s = new EdgeState();
  s->geo = Geometry{c->PMLL, c->PMLXH, c->PMLZH, c->NX, c->NZ, 2 * c->NZ * kBand + kBand * c->NX};
  std::vector<int4> tiles;
  std::vector<int> base(kSets);
  int out = 0;
  for (int set = 0; set < kSets; ++set) {
    const int n = set_count(set, c->NX, c->NZ);
    base[set] = out;
    for (int f = 0; f < n; f += kTile) {
      tiles.push_back(make_int4(set, f, std::min(kTile, n - f), out));
      out += kTile;
    }
  }
  s->ntiles = (int)tiles.size();
  s->nsamples = 0;
  for (int set = 0; set < kSets; ++set) s->nsamples += set_count(set, c->NX, c->NZ);
  int rc = FDP_OK;
  auto alloc = [&](DevArr& a, size_t bytes) {
    cudaError_t err = cudaMalloc(&a.p, bytes);
    if (err != cudaSuccess) rc = efail(e, FDP_ERR_ALLOC, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(err));
    else a.bytes = bytes;
  };
  alloc(s->tiles, tiles.size() * sizeof(int4));
  if (rc == FDP_OK) alloc(s->set_base, base.size() * sizeof(int));
  if (rc == FDP_OK) alloc(s->hist, (size_t)3 * 8 * s->geo.Rf * sizeof(float));
  if (rc == FDP_OK) alloc(s->corr, (size_t)out * kOut * sizeof(float));
  cudaError_t err = cudaSuccess;
  if (rc == FDP_OK) err = cudaMemcpyAsync(s->tiles.p, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream);
  if (rc == FDP_OK && err == cudaSuccess) err = cudaMemcpyAsync(s->set_base.p, base.data(), base.size() * sizeof(int), cudaMemcpyHostToDevice, c->stream);
  if (rc == FDP_OK && err == cudaSuccess) err = cudaMemsetAsync(s->hist.p, 0, s->hist.bytes, c->stream);
  if (rc == FDP_OK && err == cudaSuccess) err = cudaStreamSynchronize(c->stream);
  if (rc == FDP_OK && err != cudaSuccess) rc = efail(e, FDP_ERR_CUDA, "edge state: %s", cudaGetErrorString(err));
  if (rc != FDP_OK) {
    for (DevArr* a : {&s->tiles, &s->set_base, &s->hist, &s->corr}) if (a->p) cudaFree(a->p);
    delete s;
    return rc;
  }
  c->edge = s;
  *res = s;
  return FDP_OK;
}

template <int SRC> int train_tiles(fdp_edge* e, NetArgs a, int ntiles, cudaStream_t st);

NetArgs net_args(fdp_edge* e) {
  NetArgs a{};
  a.wb = (const bf16*)e->wb.p;
  a.wf = (const float*)e->w.p;
  a.scale = (const float*)e->scale.p;
  a.grad = (float*)e->g.p;
  a.loss = (double*)e->loss.p;
  a.damping = e->damping;
  return a;
}

// Sorts array samples by set into tiles; returns the order and tiles.
void array_tiles(int n, const int32_t* set, std::vector<int>& order, std::vector<int4>& tiles) {
  order.resize(n);
  for (int k = 0; k < n; ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](int p, int q) { return set[p] < set[q]; });
  tiles.clear();
  for (int k = 0; k < n;) {
    int j = k;
    while (j < n && set[order[j]] == set[order[k]] && j - k < kTile) ++j;
    tiles.push_back(make_int4(set[order[k]], k, j - k, 0));
    k = j;
  }
}

// Runs the network on host arrays (training when target != null).
int run_array(fdp_edge* e, int32_t n, const int32_t* set, const float* x, const float* target, float* y, bool train) {
  if (!e || n < 1 || !set || !x || (train && !target) || (!train && !y)) return efail(e, FDP_ERR_ARG, "bad arguments");
  for (int k = 0; k < n; ++k)
    if (set[k] < 0 || set[k] >= kSets) return efail(e, FDP_ERR_ARG, "set %d of sample %d outside 0..%d", set[k], k, kSets - 1);
  ECK(e, cudaSetDevice(e->device));
  int rc;
  if ((rc = set_smem_limits(e)) != FDP_OK) return rc;
  std::vector<int> order;
  std::vector<int4> tiles;
  array_tiles(n, set, order, tiles);
  std::vector<float> xs((size_t)n * kIn), ts(train ? (size_t)n * kOut : 0);
  for (int k = 0; k < n; ++k) {
    std::memcpy(&xs[(size_t)k * kIn], x + (size_t)order[k] * kIn, kIn * sizeof(float));
    if (train) std::memcpy(&ts[(size_t)k * kOut], target + (size_t)order[k] * kOut, kOut * sizeof(float));
  }
  if ((rc = ealloc(e, e->ax, xs.size() * sizeof(float))) || (rc = ealloc(e, e->ay, (size_t)n * kOut * sizeof(float))) ||
      (rc = ealloc(e, e->atiles, tiles.size() * sizeof(int4))) || (train && (rc = ealloc(e, e->at, ts.size() * sizeof(float)))))
    return rc;
  ECK(e, cudaMemcpyAsync(e->ax.p, xs.data(), xs.size() * sizeof(float), cudaMemcpyHostToDevice, e->stream));
  ECK(e, cudaMemcpyAsync(e->atiles.p, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice, e->stream));
  if (train) ECK(e, cudaMemcpyAsync(e->at.p, ts.data(), ts.size() * sizeof(float), cudaMemcpyHostToDevice, e->stream));
  NetArgs a = net_args(e);
  a.tiles = (const int4*)e->atiles.p;
  a.x = (const float*)e->ax.p;
  a.target = (const float*)e->at.p;
  a.y = (float*)e->ay.p;
  a.gscale = 2.f / ((float)n * kOut);
  if (train) {
    ECK(e, cudaMemsetAsync(e->loss.p, 0, sizeof(double), e->stream));
    if ((rc = train_tiles<SRC_ARRAY>(e, a, (int)tiles.size(), e->stream)) != FDP_OK) return rc;
  } else {
    k_net<SRC_ARRAY, false><<<(unsigned)tiles.size(), kTile, kSmInfer, e->stream>>>(a);
    std::vector<float> ys((size_t)n * kOut);
    ECK(e, cudaMemcpyAsync(ys.data(), e->ay.p, ys.size() * sizeof(float), cudaMemcpyDeviceToHost, e->stream));
    ECK(e, cudaStreamSynchronize(e->stream));
    for (int k = 0; k < n; ++k) std::memcpy(y + (size_t)order[k] * kOut, &ys[(size_t)k * kOut], kOut * sizeof(float));
  }
  ECK(e, cudaGetLastError());
  return FDP_OK;
}

// A training launch of the network over `ntiles` tiles and the reduction
// of their partial gradients and losses (in tile order) into the
// gradient and the loss.
template <int SRC> int train_tiles(fdp_edge* e, NetArgs a, int ntiles, cudaStream_t st) {
  int rc;
  if ((rc = ealloc(e, e->part, (size_t)ntiles * kSetP * sizeof(float))) != FDP_OK ||
      (rc = ealloc(e, e->tloss, (size_t)ntiles * sizeof(double))) != FDP_OK)
    return rc;
  a.part = (float*)e->part.p;
  a.tloss = (double*)e->tloss.p;
  k_net<SRC, true><<<(unsigned)ntiles, kTile, kSmTrain, st>>>(a);
  k_grad_reduce<<<(unsigned)((kAll + 255) / 256), 256, 0, st>>>(a.tiles, ntiles, a.part, a.tloss, a.grad, a.loss);
  ECK(e, cudaGetLastError());
  return FDP_OK;
}

int adam_step(fdp_edge* e, float lr, cudaStream_t st) {
  e->step += 1;
  const double c1 = 1.0 - std::pow(0.9, (double)e->step), c2 = 1.0 - std::pow(0.999, (double)e->step);
  k_adam<<<(unsigned)((kAll + 255) / 256), 256, 0, st>>>((float*)e->w.p, (bf16*)e->wb.p, (float*)e->m.p,
                                                          (float*)e->v.p, (float*)e->g.p, (int)kAll, lr, (float)c1,
                                                          (float)c2);
  ECK(e, cudaGetLastError());
  return FDP_OK;
}

uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ULL);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}

}  // namespace

namespace fdp {

int edge_launch(fdp_ctx* c, int it_off) {
  EdgeState* s = c->edge;
  if (!s || !s->net || !c->edge_attached) return 0;
  fdp_edge* e = s->net;
  NetArgs a = net_args(e);
  a.tiles = (const int4*)s->tiles.p;
  a.y = (float*)s->corr.p;
  a.t = view_of(c);
  a.hist = (const float*)s->hist.p;
  a.geo = s->geo;
  a.it_base = (const int*)c->itbase.p;
  a.it_off = it_off;
  k_net<SRC_BAND, false><<<s->ntiles, kTile, kSmInfer, c->stream>>>(a);
  const int maxn = std::max(c->NZ, c->NX);
  for (int c0 : {0, kDepth})
    k_edge_commit<<<dim3((maxn + 127) / 128, c0 == 0 ? kDepth : kBand - kDepth, 3), 128, 0, c->stream>>>(
        a.t, s->geo, (float*)s->hist.p, (const float*)s->corr.p, (const int*)s->set_base.p,
        (const float*)e->scale.p, (const int*)c->itbase.p, it_off, c0, e->damping);
  return 3;
}

void edge_release(fdp_ctx* c) {
  EdgeState* s = c->edge;
  if (!s) return;
  for (DevArr* a : {&s->tiles, &s->set_base, &s->hist, &s->corr}) if (a->p) cudaFree(a->p);
  delete s;
  c->edge = nullptr;
  c->edge_attached = false;
}

}  // namespace fdp

extern "C" {

int fdp_edge_create(int32_t device, const float* scale8, uint64_t seed, fdp_edge** out) {
  if (!out) return efail(nullptr, FDP_ERR_ARG, "null output");
  *out = nullptr;
  fdp_edge* e = new fdp_edge();
  e->device = device;
  auto bail = [&](int rc) { g_edge_error = e->err; fdp_edge_destroy(e); return rc; };
  cudaError_t err = cudaSetDevice(device);
  if (err == cudaSuccess) err = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking);
  if (err != cudaSuccess) return bail(efail(e, FDP_ERR_CUDA, "edge stream: %s", cudaGetErrorString(err)));
  int rc;
  if ((rc = ealloc(e, e->w, kAll * 4)) || (rc = ealloc(e, e->wb, kAll * 2)) || (rc = ealloc(e, e->m, kAll * 4)) ||
      (rc = ealloc(e, e->v, kAll * 4)) || (rc = ealloc(e, e->g, kAll * 4)) || (rc = ealloc(e, e->scale, 8 * 4)) ||
      (rc = ealloc(e, e->loss, sizeof(double))))
    return bail(rc);
  // uniform +-1/sqrt(fan-in) hidden weights, zero biases and output layer
  std::vector<float> w(kAll, 0.f);
  uint64_t st = seed;
  for (int set = 0; set < kSets; ++set) {
    float* p = &w[(size_t)set * kSetP];
    for (int k = 0; k < kHid * kIn; ++k) p[oW1 + k] = (float)(((splitmix(st) >> 11) * 0x1.0p-53 * 2.0 - 1.0) / std::sqrt((double)kIn));
    for (int k = 0; k < kHid * kHid; ++k) p[oW2 + k] = (float)(((splitmix(st) >> 11) * 0x1.0p-53 * 2.0 - 1.0) / std::sqrt((double)kHid));
  }
  if (scale8) std::memcpy(e->hscale, scale8, sizeof e->hscale);
  for (float sc : e->hscale)
    if (!(sc > 0.f)) return bail(efail(e, FDP_ERR_ARG, "field scales must be positive"));
  err = cudaMemcpyAsync(e->w.p, w.data(), kAll * 4, cudaMemcpyHostToDevice, e->stream);
  if (err == cudaSuccess) err = cudaMemsetAsync(e->m.p, 0, kAll * 4, e->stream);
  if (err == cudaSuccess) err = cudaMemsetAsync(e->v.p, 0, kAll * 4, e->stream);
  if (err == cudaSuccess) err = cudaMemsetAsync(e->g.p, 0, kAll * 4, e->stream);
  if (err != cudaSuccess) return bail(efail(e, FDP_ERR_CUDA, "edge init: %s", cudaGetErrorString(err)));
  if ((rc = refresh_bf16(e)) || (rc = sync_scale(e))) return bail(rc);
  *out = e;
  return FDP_OK;
}

int fdp_edge_get_params(fdp_edge* e, float* params) {
  if (!e || !params) return efail(e, FDP_ERR_ARG, "null argument");
  ECK(e, cudaSetDevice(e->device));
  ECK(e, cudaMemcpyAsync(params, e->w.p, kAll * 4, cudaMemcpyDeviceToHost, e->stream));
  ECK(e, cudaStreamSynchronize(e->stream));
  return FDP_OK;
}

int fdp_edge_set_params(fdp_edge* e, const float* params) {
  if (!e || !params) return efail(e, FDP_ERR_ARG, "null argument");
  ECK(e, cudaSetDevice(e->device));
  ECK(e, cudaMemcpyAsync(e->w.p, params, kAll * 4, cudaMemcpyHostToDevice, e->stream));
  ECK(e, cudaMemsetAsync(e->m.p, 0, kAll * 4, e->stream));
  ECK(e, cudaMemsetAsync(e->v.p, 0, kAll * 4, e->stream));
  ECK(e, cudaMemsetAsync(e->g.p, 0, kAll * 4, e->stream));
  e->step = 0;
  int rc = refresh_bf16(e);
  if (rc != FDP_OK) return rc;
  ECK(e, cudaStreamSynchronize(e->stream));
  return FDP_OK;
}

int fdp_edge_set_output(fdp_edge* e, int32_t kind) {
  if (!e || (kind != FDP_EDGE_CORRECT && kind != FDP_EDGE_DAMP)) return efail(e, FDP_ERR_ARG, "bad output kind");
  e->damping = kind == FDP_EDGE_DAMP;
  return FDP_OK;
}

int fdp_edge_get_scale(fdp_edge* e, float* scale8) {
  if (!e || !scale8) return efail(e, FDP_ERR_ARG, "null argument");
  std::memcpy(scale8, e->hscale, sizeof e->hscale);
  return FDP_OK;
}

int fdp_edge_set_scale(fdp_edge* e, const float* scale8) {
  if (!e || !scale8) return efail(e, FDP_ERR_ARG, "null argument");
  for (int f = 0; f < 8; ++f)
    if (!(scale8[f] > 0.f)) return efail(e, FDP_ERR_ARG, "field scales must be positive");
  std::memcpy(e->hscale, scale8, sizeof e->hscale);
  ECK(e, cudaSetDevice(e->device));
  return sync_scale(e);
}

int fdp_edge_forward(fdp_edge* e, int32_t n, const int32_t* set, const float* x, float* y) {
  return run_array(e, n, set, x, nullptr, y, false);
}

int fdp_edge_gradients(fdp_edge* e, int32_t n, const int32_t* set, const float* x, const float* target, float* grad,
                       double* loss) {
  if (!grad) return efail(e, FDP_ERR_ARG, "null gradient output");
  int rc = run_array(e, n, set, x, target, nullptr, true);
  if (rc != FDP_OK) return rc;
  double se = 0.0;
  ECK(e, cudaMemcpyAsync(grad, e->g.p, kAll * 4, cudaMemcpyDeviceToHost, e->stream));
  ECK(e, cudaMemcpyAsync(&se, e->loss.p, sizeof se, cudaMemcpyDeviceToHost, e->stream));
  ECK(e, cudaMemsetAsync(e->g.p, 0, kAll * 4, e->stream));
  ECK(e, cudaStreamSynchronize(e->stream));
  if (loss) *loss = se / ((double)n * kOut);
  return FDP_OK;
}

int fdp_edge_train_batch(fdp_edge* e, int32_t n, const int32_t* set, const float* x, const float* target, float lr,
                         double* loss) {
  int rc = run_array(e, n, set, x, target, nullptr, true);
  if (rc != FDP_OK) return rc;
  if ((rc = adam_step(e, lr, e->stream)) != FDP_OK) return rc;
  double se = 0.0;
  ECK(e, cudaMemcpyAsync(&se, e->loss.p, sizeof se, cudaMemcpyDeviceToHost, e->stream));
  ECK(e, cudaStreamSynchronize(e->stream));
  if (loss) *loss = se / ((double)n * kOut);
  return FDP_OK;
}

int fdp_edge_train_level(fdp_edge* e, fdp_ctx* trunc, fdp_ctx* ext, int32_t ox, int32_t level, float lr,
                         int32_t teacher, double* loss) {
  const TraceRange trace("fdp_edge_train_level");
  if (!e || !trunc || !ext) return efail(e, FDP_ERR_ARG, "null argument");
  if (trunc->prec != 4 || ext->prec != 4) return efail(e, FDP_ERR_UNSUPPORTED, "the learned edge runs on FP32 contexts");
  if ((trunc->g.stress_imaging != 0) != (ext->g.stress_imaging != 0))
    return efail(e, FDP_ERR_ARG, "the two contexts differ in free-surface mode");
  if (trunc->PMLL + ox < 1 || trunc->PMLXH + ox > ext->MX || trunc->PMLZH > ext->MZ)
    return efail(e, FDP_ERR_ARG, "the target's interior does not hold the context's grid at column offset %d", ox);
  if (trunc->edge_attached) return efail(e, FDP_ERR_STATE, "detach the edge before training on this context");
  if (level < 1) return efail(e, FDP_ERR_ARG, "level must be >= 1");
  ECK(e, cudaSetDevice(e->device));
  int rc;
  if ((rc = set_smem_limits(e)) != FDP_OK) return rc;
  EdgeState* s = nullptr;
  if ((rc = edge_state(e, trunc, &s)) != FDP_OK) return rc;
  cudaEvent_t ev;
  ECK(e, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
  ECK(e, cudaEventRecord(ev, ext->stream));
  ECK(e, cudaStreamWaitEvent(trunc->stream, ev, 0));
  NetArgs a = net_args(e);
  a.tiles = (const int4*)s->tiles.p;
  a.t = view_of(trunc);
  a.e = view_of(ext);
  a.ox = ox;
  a.hist = (const float*)s->hist.p;
  a.geo = s->geo;
  a.it_base = nullptr;
  a.it_off = level;
  a.gscale = 2.f / ((float)s->nsamples * kOut);
  a.y = teacher ? nullptr : (float*)s->corr.p;
  ECK(e, cudaMemsetAsync(e->loss.p, 0, sizeof(double), trunc->stream));
  if ((rc = train_tiles<SRC_BAND>(e, a, s->ntiles, trunc->stream)) != FDP_OK) return rc;
  if ((rc = adam_step(e, lr, trunc->stream)) != FDP_OK) return rc;
  if (teacher) {
    k_edge_teacher<<<dim3((trunc->NX + 127) / 128, trunc->NZ, 1), 128, 0, trunc->stream>>>(a.t, a.e, ox, s->geo,
                                                                                          (float*)s->hist.p, level);
  } else {
    // the correction the network gave before this step, applied as in a run
    const int maxn = std::max(trunc->NZ, trunc->NX);
    for (int c0 : {0, kDepth})
      k_edge_commit<<<dim3((maxn + 127) / 128, c0 == 0 ? kDepth : kBand - kDepth, 3), 128, 0, trunc->stream>>>(
          a.t, s->geo, (float*)s->hist.p, (const float*)s->corr.p, (const int*)s->set_base.p,
          (const float*)e->scale.p, nullptr, level, c0, e->damping);
  }
  ECK(e, cudaGetLastError());
  ECK(e, cudaEventRecord(ev, trunc->stream));
  ECK(e, cudaStreamWaitEvent(ext->stream, ev, 0));
  cudaEventDestroy(ev);
  if (loss) {
    double se = 0.0;
    ECK(e, cudaMemcpyAsync(&se, e->loss.p, sizeof se, cudaMemcpyDeviceToHost, trunc->stream));
    ECK(e, cudaStreamSynchronize(trunc->stream));
    *loss = se / ((double)s->nsamples * kOut);
  }
  return FDP_OK;
}

int fdp_edge_attach(fdp_ctx* trunc, fdp_edge* e) {
  if (!trunc) return efail(e, FDP_ERR_ARG, "null context");
  if (!e) {
    fdp::edge_release(trunc);
  } else {
    ECK(e, cudaSetDevice(e->device));
    int rc;
    if ((rc = set_smem_limits(e)) != FDP_OK) return rc;
    fdp::edge_release(trunc);  // history starts at rest
    EdgeState* s = nullptr;
    if ((rc = edge_state(e, trunc, &s)) != FDP_OK) return rc;
    s->net = e;
    trunc->edge_attached = true;
  }
  params_changed(trunc);  // the captured graph gains or loses the edge kernels
  return FDP_OK;
}

const char* fdp_edge_last_error(const fdp_edge* e) { return e ? e->err.c_str() : g_edge_error.c_str(); }

void fdp_edge_destroy(fdp_edge* e) {
  if (!e) return;
  if (e->stream) cudaStreamSynchronize(e->stream);
  for (DevArr* a : {&e->w, &e->wb, &e->m, &e->v, &e->g, &e->scale, &e->loss, &e->ax, &e->at, &e->ay, &e->atiles,
                    &e->part, &e->tloss})
    if (a->p) cudaFree(a->p);
  if (e->stream) cudaStreamDestroy(e->stream);
  delete e;
}

}  // extern "C"
