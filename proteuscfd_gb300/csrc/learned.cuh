// Learned right preconditioner: device kernels of the edge message-passing
// network (included into solver.cu inside its anonymous namespace).
//
// The preconditioner has no reference counterpart; it sits where
// CRS<T>::PrecondBackSolve sits (ucs/crs.tcc:591).  Network (sizes and the
// parameter layout are fixed by the PCFD_LP_* constants of pcfd.h):
//   h0   = ReLU(Win x + bin)                                   11 -> 64
//   m_i  = (1/deg_i) sum_j (We e_ij + ce) * h_j   (per channel)
//   h'   = ReLU(Ws h + Wm m + b)                               128 -> 64, x3
//   out  = Wout h3 + bout                                      64 -> 5
// Matrices are BF16 (rounded from the FP32 master copy), biases and all
// accumulation FP32, activations h and m stored BF16.  The 128-row layer
// products [h | m] (128 x 128) x [Ws | Wm]^T (128 x 64) and, in the backward
// pass, dz (128 x 64) x [Ws | Wm] (64 x 128) run on the tensor cores
// (tcgen05.mma, accumulator in TMEM); the weight image reaches shared memory
// through the bulk copy engine.  Gathers, the encoder, the decoder and the
// weight gradients run on the FP32 pipes.
#pragma once

#include "umma.cuh"

constexpr int LP_NIN = PCFD_LP_NIN;
constexpr int LP_H = PCFD_LP_HIDDEN;
constexpr int LP_NE = PCFD_LP_NEDGE;
constexpr int LP_NOUT = PCFD_LP_NOUT;
constexpr int LP_NL = PCFD_LP_LAYERS;
constexpr int LP_OFF_WIN = 0;
constexpr int LP_OFF_BIN = LP_H * LP_NIN;
constexpr int LP_OFF_L0 = LP_OFF_BIN + LP_H;
constexpr int LP_L_WE = 0;
constexpr int LP_L_CE = LP_H * LP_NE;
constexpr int LP_L_WS = LP_L_CE + LP_H;
constexpr int LP_L_WM = LP_L_WS + LP_H * LP_H;
constexpr int LP_L_B = LP_L_WM + LP_H * LP_H;
constexpr int LP_L_SIZE = LP_L_B + LP_H;
constexpr int LP_OFF_WOUT = LP_OFF_L0 + LP_NL * LP_L_SIZE;
constexpr int LP_OFF_BOUT = LP_OFF_WOUT + LP_NOUT * LP_H;
constexpr int LP_NPARAM = LP_OFF_BOUT + LP_NOUT;
static_assert(LP_NPARAM == PCFD_LP_NPARAM, "parameter layout");

constexpr int LP_TILE = 128;                        // nodes per CTA (MMA M)
constexpr int LP_THREADS = 256;                     // 8 warps
constexpr int LP_IMG = LP_H * 2 * LP_H;             // BF16 values in one weight image (64 x 128)
constexpr uint32_t LP_IMG_BYTES = LP_IMG * 2;       // 16 KiB
constexpr int LP_ERR_TIMEOUT = 1;

// shared memory of the layer kernels: A tile, weight image, barriers
constexpr size_t LP_SMEM_A = (size_t)LP_TILE * 2 * LP_H * 2;  // 32 KiB
constexpr size_t LP_SMEM = 1024 + LP_SMEM_A + LP_IMG_BYTES + 64;

__device__ __forceinline__ float bfr(float v) { return __bfloat162float(__float2bfloat16(v)); }

struct LpSmem {
  unsigned char* a;   // A operand tile (K-major canonical)
  unsigned char* b;   // weight image
  uint64_t* bar_w;    // bulk-copy completion
  uint64_t* bar_mma;  // MMA completion
  uint32_t* tmem_holder;
};
__device__ __forceinline__ LpSmem lp_smem(unsigned char* raw) {
  uintptr_t base = (reinterpret_cast<uintptr_t>(raw) + 1023) & ~uintptr_t(1023);
  LpSmem s;
  s.a = reinterpret_cast<unsigned char*>(base);
  s.b = s.a + LP_SMEM_A;
  s.bar_w = reinterpret_cast<uint64_t*>(s.b + LP_IMG_BYTES);
  s.bar_mma = s.bar_w + 1;
  s.tmem_holder = reinterpret_cast<uint32_t*>(s.bar_mma + 1);
  return s;
}

// Start of a layer kernel: barriers, the weight image copy, TMEM columns.
__device__ __forceinline__ void lp_begin(const LpSmem& sm, const __nv_bfloat16* img, uint32_t ncols) {
  const int tid = threadIdx.x;
  if (tid == 0) {
    umma::mbar_init(sm.bar_w, 1);
    umma::mbar_init(sm.bar_mma, 1);
    umma::fence_mbar_init();
  }
  __syncthreads();
  if (tid == 0) {
    umma::mbar_expect_tx(sm.bar_w, LP_IMG_BYTES);
    umma::bulk_g2s(sm.b, img, LP_IMG_BYTES, sm.bar_w);
  }
  if ((tid >> 5) == 0) umma::tmem_alloc(sm.tmem_holder, ncols);
}

// After the A tile is written: one thread issues the K/16 MMAs and commits.
// Returns the TMEM address; *ok is false when a bounded wait expired.
template <int K, int N>
__device__ __forceinline__ uint32_t lp_mma(const LpSmem& sm, bool* ok) {
  umma::fence_async_smem();
  umma::fence_before_sync();
  __syncthreads();
  umma::fence_after_sync();
  const uint32_t tmem = *sm.tmem_holder;
  bool good = true;
  if (threadIdx.x == 0) {
    good = umma::mbar_wait(sm.bar_w, 0);
    if (good) {
      constexpr uint32_t idesc = umma::idesc_bf16(LP_TILE, N);
      const uint32_t a0 = umma::smem_addr(sm.a), b0 = umma::smem_addr(sm.b);
#pragma unroll
      for (int ks = 0; ks < K / 16; ks++) {
        const uint64_t ad = umma::smem_desc(a0 + ks * 256, 128, (K / 8) * 128);
        const uint64_t bd = umma::smem_desc(b0 + ks * 256, 128, (K / 8) * 128);
        umma::mma_bf16(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
      }
      umma::mma_commit(sm.bar_mma);
    }
  }
  // every thread waits (bounded) for the accumulator
  good = __syncthreads_and(good ? 1 : 0) != 0;
  if (good) good = umma::mbar_wait(sm.bar_mma, 0);
  umma::fence_after_sync();
  *ok = good;
  return tmem;
}

__device__ __forceinline__ void lp_end(uint32_t tmem, uint32_t ncols) {
  umma::fence_before_sync();
  __syncthreads();
  if ((threadIdx.x >> 5) == 0) umma::tmem_dealloc(tmem, ncols);
}

// gate of channel pair (c, c+1) for edge features e seen with normal sign sg
struct Gate2 {
  float w0[4], w1[4], c0, c1;
};
__device__ __forceinline__ Gate2 load_gate(const float* __restrict__ wl, int c) {
  Gate2 g;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    g.w0[k] = bfr(wl[LP_L_WE + c * LP_NE + k]);
    g.w1[k] = bfr(wl[LP_L_WE + (c + 1) * LP_NE + k]);
  }
  g.c0 = wl[LP_L_CE + c];
  g.c1 = wl[LP_L_CE + c + 1];
  return g;
}
__device__ __forceinline__ float2 gate_eval(const Gate2& g, float4 e, float sg) {
  float2 r;
  r.x = fmaf(g.w0[3], e.w, fmaf(g.w0[2], sg * e.z, fmaf(g.w0[1], sg * e.y, fmaf(g.w0[0], sg * e.x, g.c0))));
  r.y = fmaf(g.w1[3], e.w, fmaf(g.w1[2], sg * e.z, fmaf(g.w1[1], sg * e.y, fmaf(g.w1[0], sg * e.x, g.c1))));
  return r;
}

__device__ __forceinline__ void st_a2(unsigned char* a, int r, int k, int K, __nv_bfloat162 v) {
  *reinterpret_cast<__nv_bfloat162*>(a + umma::tile_offset(r, k, K)) = v;
}

// ---------------------------------------------------------------------------
// forward
// ---------------------------------------------------------------------------

// node features (pcfd_lp_features): y/sigma, state, log volume
__global__ void k_lp_features(int n, const double* __restrict__ y, const double* __restrict__ sigma_dev,
                              const double* __restrict__ q, const double* __restrict__ vol, double rho_inf,
                              double p_inf, double c_inf, double vmean, float* __restrict__ x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double sigma = *sigma_dev;
  const double isig = sigma > 0.0 ? 1.0 / sigma : 0.0;
  const double* Q = &q[(size_t)i * NVARS];
  float* xi = &x[(size_t)i * LP_NIN];
#pragma unroll
  for (int k = 0; k < 5; k++) xi[k] = (float)(y[(size_t)i * 5 + k] * isig);
  xi[5] = (float)(Q[0] / rho_inf - 1.0);
  xi[6] = (float)(Q[7] / c_inf);
  xi[7] = (float)(Q[8] / c_inf);
  xi[8] = (float)(Q[9] / c_inf);
  xi[9] = (float)(Q[6] / p_inf - 1.0);
  xi[10] = (float)log(vol[i] / vmean);
}

// sigma = sqrt(sum / count) from the k_sumsq partials
__global__ void k_lp_sigma(int nparts, const double* __restrict__ part, double count, double* __restrict__ sigma) {
  __shared__ double red[256];
  double a = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) a += part[i];
  red[threadIdx.x] = a;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *sigma = sqrt(red[0] / count);
}

// encoder: one thread per (node, channel pair)
__global__ void k_lp_encode(int n, const float* __restrict__ x, const float* __restrict__ w,
                            __nv_bfloat16* __restrict__ h0) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)n * (LP_H / 2)) return;
  const int i = (int)(t / (LP_H / 2));
  const int c = (int)(t % (LP_H / 2)) * 2;
  float a0 = w[LP_OFF_BIN + c], a1 = w[LP_OFF_BIN + c + 1];
#pragma unroll
  for (int k = 0; k < LP_NIN; k++) {
    const float xv = x[(size_t)i * LP_NIN + k];
    a0 = fmaf(bfr(w[LP_OFF_WIN + c * LP_NIN + k]), xv, a0);
    a1 = fmaf(bfr(w[LP_OFF_WIN + (c + 1) * LP_NIN + k]), xv, a1);
  }
  *reinterpret_cast<__nv_bfloat162*>(&h0[(size_t)i * LP_H + c]) =
      __floats2bfloat162_rn(fmaxf(a0, 0.f), fmaxf(a1, 0.f));
}

// Packed FP32 fused multiply-add of two lanes (PTX fma.rn.f32x2): each half
// is rounded as fmaf rounds it.
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  uint64_t d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;"
      : "=l"(d)
      : "l"(*reinterpret_cast<const uint64_t*>(&a)), "l"(*reinterpret_cast<const uint64_t*>(&b)),
        "l"(*reinterpret_cast<const uint64_t*>(&c)));
  return *reinterpret_cast<const float2*>(&d);
}

// m for one block of up to 32 neighbours of a row: lane k holds the k-th
// neighbour's index jl and edge features el; cnt of them are valid.  The row
// loads of 16 neighbours are issued together, then summed in neighbour order
// (the order of the sequential sum).  The channel pair's gate and sum use
// packed FMAs: the same operations and roundings as gate_eval(g, e, 1) and
// two fmaf, in half the instructions.  The per-neighbour branch stays: the
// branch-free form (zero rows in the padded slots) measured twice as slow,
// with the row loads no longer in flight together.
__device__ __forceinline__ void lp_gather_block(const Gate2& g, const __nv_bfloat16* __restrict__ h_in, int c,
                                                int jl, float4 el, int cnt, float& a0, float& a1) {
  const float2 w0 = make_float2(g.w0[0], g.w1[0]), w1 = make_float2(g.w0[1], g.w1[1]);
  const float2 w2 = make_float2(g.w0[2], g.w1[2]), w3 = make_float2(g.w0[3], g.w1[3]);
  const float2 c0 = make_float2(g.c0, g.c1);
  float2 acc = make_float2(a0, a1);
  for (int t = 0; t < cnt; t += 16) {
    uint32_t raw[16];
#pragma unroll
    for (int u = 0; u < 16; u++) {
      const int j = __shfl_sync(0xffffffffu, jl, t + u);
      raw[u] = 0u;
      if (t + u < cnt) raw[u] = *reinterpret_cast<const uint32_t*>(&h_in[(size_t)j * LP_H + c]);
    }
#pragma unroll
    for (int u = 0; u < 16; u++) {
      float4 e;
      e.x = __shfl_sync(0xffffffffu, el.x, t + u);
      e.y = __shfl_sync(0xffffffffu, el.y, t + u);
      e.z = __shfl_sync(0xffffffffu, el.z, t + u);
      e.w = __shfl_sync(0xffffffffu, el.w, t + u);
      if (t + u < cnt) {
        const float2 hh = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&raw[u]));
        float2 gv = fma2(w0, make_float2(e.x, e.x), c0);
        gv = fma2(w1, make_float2(e.y, e.y), gv);
        gv = fma2(w2, make_float2(e.z, e.z), gv);
        gv = fma2(w3, make_float2(e.w, e.w), gv);
        acc = fma2(gv, hh, acc);
      }
    }
  }
  a0 = acc.x;
  a1 = acc.y;
}

// One message-passing layer for 128 nodes.  Gather phase: warp w builds rows
// 16w..16w+15 of A = [h | m]; lane l owns channels 2l, 2l+1.  The warp's row
// pointers arrive in one load; a row's neighbour indices and edge features
// arrive in one coalesced load, issued while the previous row's neighbour rows
// are gathered; 16 neighbour rows are in flight at once.  Then one 128x64x128
// MMA, and the epilogue (warps 0-3, one row per thread, TMEM read 16 columns at
// a time) adds the bias, applies ReLU and stores h' in BF16; the last layer
// also applies the decoder and writes either out (FP32) or z = y + sigma * out
// (FP64).  80 registers: three CTAs per multiprocessor.
template <bool LAST>
__global__ void __launch_bounds__(LP_THREADS, 3) k_lp_layer(
    int n, const int* __restrict__ nptr, const int* __restrict__ nnbr, const float4* __restrict__ ef,
    const float* __restrict__ invdeg, const __nv_bfloat16* __restrict__ h_in, const float* __restrict__ wl,
    const __nv_bfloat16* __restrict__ img, __nv_bfloat16* __restrict__ h_out, __nv_bfloat16* __restrict__ m_out,
    const float* __restrict__ w, float* __restrict__ out, const double* __restrict__ y,
    const double* __restrict__ sigma_dev, double* __restrict__ z, int* __restrict__ err) {
  extern __shared__ unsigned char lp_raw[];
  const LpSmem sm = lp_smem(lp_raw);
  constexpr int K = 2 * LP_H;
  constexpr int RPW = LP_TILE / 8;  // rows per warp
  lp_begin(sm, img, LP_H);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int c = 2 * lane;
  const int base = blockIdx.x * LP_TILE;
  const int r0 = warp * RPW;
  {
    const Gate2 g = load_gate(wl, c);
    // lane k <= RPW holds nptr of row r0 + k (nptr has n + 1 entries)
    int pl = 0;
    if (lane <= RPW && base + r0 + lane <= n) pl = nptr[base + r0 + lane];
    // the first 32 neighbours of row rr: index and edge features
    auto fetch = [&](int rr, int& jl, float4& el) {
      const int p0 = __shfl_sync(0xffffffffu, pl, rr), p1 = __shfl_sync(0xffffffffu, pl, rr + 1);
      jl = 0;
      el = make_float4(0.f, 0.f, 0.f, 0.f);
      if (base + r0 + rr < n && lane < p1 - p0) {
        jl = nnbr[p0 + lane];
        el = ef[p0 + lane];
      }
    };
    int jl;
    float4 el;
    fetch(0, jl, el);
    for (int rr = 0; rr < RPW; rr++) {
      int jn = 0;
      float4 en = make_float4(0.f, 0.f, 0.f, 0.f);
      if (rr + 1 < RPW) fetch(rr + 1, jn, en);
      const int r = r0 + rr;
      const int i = base + r;
      __nv_bfloat162 hv = __floats2bfloat162_rn(0.f, 0.f), mv = hv;
      if (i < n) {
        const int p0 = __shfl_sync(0xffffffffu, pl, rr), p1 = __shfl_sync(0xffffffffu, pl, rr + 1);
        hv = *reinterpret_cast<const __nv_bfloat162*>(&h_in[(size_t)i * LP_H + c]);
        float a0 = 0.f, a1 = 0.f;
        lp_gather_block(g, h_in, c, jl, el, min(p1 - p0, 32), a0, a1);
        // rows with more than 32 neighbours
        for (int pb = p0 + 32; pb < p1; pb += 32) {
          int jx = 0;
          float4 ex = make_float4(0.f, 0.f, 0.f, 0.f);
          if (lane < p1 - pb) {
            jx = nnbr[pb + lane];
            ex = ef[pb + lane];
          }
          lp_gather_block(g, h_in, c, jx, ex, min(p1 - pb, 32), a0, a1);
        }
        const float id = invdeg[i];
        mv = __floats2bfloat162_rn(a0 * id, a1 * id);
        if (m_out) *reinterpret_cast<__nv_bfloat162*>(&m_out[(size_t)i * LP_H + c]) = mv;
      }
      st_a2(sm.a, r, c, K, hv);
      st_a2(sm.a, r, LP_H + c, K, mv);
      jl = jn;
      el = en;
    }
  }
  bool ok;
  const uint32_t tmem = lp_mma<K, LP_H>(sm, &ok);
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(err, LP_ERR_TIMEOUT);
  } else if (warp < 4) {
    const int r = warp * 32 + lane;
    const int i = base + r;
    float o[LP_NOUT];
#pragma unroll
    for (int oo = 0; oo < LP_NOUT; oo++) o[oo] = LAST ? w[LP_OFF_BOUT + oo] : 0.f;
#pragma unroll
    for (int cc = 0; cc < LP_H; cc += 16) {
      float v[16];
      umma::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + cc, v);
      if (i < n) {
#pragma unroll
        for (int k = 0; k < 16; k++) v[k] = bfr(fmaxf(v[k] + wl[LP_L_B + cc + k], 0.f));
        if (!LAST || h_out) {
          uint4* dst = reinterpret_cast<uint4*>(&h_out[(size_t)i * LP_H + cc]);
#pragma unroll
          for (int q8 = 0; q8 < 2; q8++) {
            __nv_bfloat162 b0 = __floats2bfloat162_rn(v[8 * q8], v[8 * q8 + 1]);
            __nv_bfloat162 b1 = __floats2bfloat162_rn(v[8 * q8 + 2], v[8 * q8 + 3]);
            __nv_bfloat162 b2 = __floats2bfloat162_rn(v[8 * q8 + 4], v[8 * q8 + 5]);
            __nv_bfloat162 b3 = __floats2bfloat162_rn(v[8 * q8 + 6], v[8 * q8 + 7]);
            uint4 u;
            u.x = *reinterpret_cast<uint32_t*>(&b0);
            u.y = *reinterpret_cast<uint32_t*>(&b1);
            u.z = *reinterpret_cast<uint32_t*>(&b2);
            u.w = *reinterpret_cast<uint32_t*>(&b3);
            dst[q8] = u;
          }
        }
        if (LAST) {
#pragma unroll
          for (int oo = 0; oo < LP_NOUT; oo++)
#pragma unroll
            for (int k = 0; k < 16; k++) o[oo] = fmaf(bfr(w[LP_OFF_WOUT + oo * LP_H + cc + k]), v[k], o[oo]);
        }
      }
    }
    if (LAST && i < n) {
      if (out) {
#pragma unroll
        for (int oo = 0; oo < LP_NOUT; oo++) out[(size_t)i * LP_NOUT + oo] = o[oo];
      }
      if (z) {
        const double sg = *sigma_dev;
#pragma unroll
        for (int oo = 0; oo < LP_NOUT; oo++) z[(size_t)i * 5 + oo] = y[(size_t)i * 5 + oo] + sg * (double)o[oo];
      }
    }
  }
  lp_end(tmem, LP_H);
}

// ---------------------------------------------------------------------------
// backward
// ---------------------------------------------------------------------------

// per-block partial sums -> gradient slice (fixed order: deterministic)
__global__ void k_lp_reduce(int nblk, int len, const float* __restrict__ part, float* __restrict__ grad) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= len) return;
  float a = 0.f;
  for (int b = 0; b < nblk; b++) a += part[(size_t)b * len + k];
  grad[k] = a;
}

// block-wide sum of per-warp arrays in shared memory: red[warp][len] -> out
__device__ __forceinline__ void lp_block_sum(float* red, int len, float* out) {
  __syncthreads();
  for (int k = threadIdx.x; k < len; k += blockDim.x) {
    float a = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) a += red[w * len + k];
    out[k] = a;
  }
}

// decoder backward: dout = 2 (out - t) / (5 n); dh3 = Wout^T dout; partials
// of dWout, dbout and the loss.  Warp per node stripe, lane = channel pair.
constexpr int LP_DEC_LEN = LP_NOUT * LP_H + LP_NOUT + 1;
__global__ void __launch_bounds__(256) k_lp_dec_bwd(int n, const float* __restrict__ out, const float* __restrict__ t,
                                                    const __nv_bfloat16* __restrict__ h3, const float* __restrict__ w,
                                                    float* __restrict__ dh, float* __restrict__ part) {
  __shared__ float red[8 * LP_DEC_LEN];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, c = 2 * lane;
  const float scale = 2.0f / (5.0f * (float)n);
  float gw0[LP_NOUT] = {0}, gw1[LP_NOUT] = {0}, gb[LP_NOUT] = {0}, gl = 0.f;
  float wo0[LP_NOUT], wo1[LP_NOUT];
#pragma unroll
  for (int o = 0; o < LP_NOUT; o++) {
    wo0[o] = bfr(w[LP_OFF_WOUT + o * LP_H + c]);
    wo1[o] = bfr(w[LP_OFF_WOUT + o * LP_H + c + 1]);
  }
  const int nwarps = gridDim.x * (blockDim.x >> 5);
  for (int i = blockIdx.x * (blockDim.x >> 5) + warp; i < n; i += nwarps) {
    float d[LP_NOUT];
#pragma unroll
    for (int o = 0; o < LP_NOUT; o++) {
      const float r = out[(size_t)i * LP_NOUT + o] - t[(size_t)i * LP_NOUT + o];
      d[o] = scale * r;
      gl = fmaf(r, r, gl);
      gb[o] += d[o];
    }
    const float2 hv = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&h3[(size_t)i * LP_H + c]));
    float a0 = 0.f, a1 = 0.f;
#pragma unroll
    for (int o = 0; o < LP_NOUT; o++) {
      a0 = fmaf(wo0[o], d[o], a0);
      a1 = fmaf(wo1[o], d[o], a1);
      gw0[o] = fmaf(d[o], hv.x, gw0[o]);
      gw1[o] = fmaf(d[o], hv.y, gw1[o]);
    }
    *reinterpret_cast<float2*>(&dh[(size_t)i * LP_H + c]) = make_float2(a0, a1);
  }
  float* my = red + warp * LP_DEC_LEN;
#pragma unroll
  for (int o = 0; o < LP_NOUT; o++) {
    my[o * LP_H + c] = gw0[o];
    my[o * LP_H + c + 1] = gw1[o];
  }
  if (lane == 0) {
#pragma unroll
    for (int o = 0; o < LP_NOUT; o++) my[LP_NOUT * LP_H + o] = gb[o];
  }
  // loss: sum over lanes is 32x the node sum (every lane saw every node)
  if (lane == 0) my[LP_NOUT * LP_H + LP_NOUT] = gl;
  lp_block_sum(red, LP_DEC_LEN, part + (size_t)blockIdx.x * LP_DEC_LEN);
}

// Layer backward on the tensor cores: dz = BF16(dh * (h' > 0)) (stored for
// the weight gradients), then [dh_self | dm] = dz x [Ws | Wm] (128 x 128).
__global__ void __launch_bounds__(LP_THREADS) k_lp_layer_bwd(int n, const float* __restrict__ dh,
                                                             const __nv_bfloat16* __restrict__ h_out,
                                                             const __nv_bfloat16* __restrict__ img,
                                                             __nv_bfloat16* __restrict__ dz_out,
                                                             float* __restrict__ dh_self, float* __restrict__ dm,
                                                             int* __restrict__ err) {
  extern __shared__ unsigned char lp_raw[];
  const LpSmem sm = lp_smem(lp_raw);
  constexpr int K = LP_H;
  lp_begin(sm, img, 2 * LP_H);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, c = 2 * lane;
  const int base = blockIdx.x * LP_TILE;
  for (int rr = 0; rr < LP_TILE / 8; rr++) {
    const int r = warp * (LP_TILE / 8) + rr;
    const int i = base + r;
    __nv_bfloat162 dv = __floats2bfloat162_rn(0.f, 0.f);
    if (i < n) {
      const float2 d = *reinterpret_cast<const float2*>(&dh[(size_t)i * LP_H + c]);
      const float2 hv = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&h_out[(size_t)i * LP_H + c]));
      dv = __floats2bfloat162_rn(hv.x > 0.f ? d.x : 0.f, hv.y > 0.f ? d.y : 0.f);
      *reinterpret_cast<__nv_bfloat162*>(&dz_out[(size_t)i * LP_H + c]) = dv;
    }
    st_a2(sm.a, r, c, K, dv);
  }
  bool ok;
  const uint32_t tmem = lp_mma<K, 2 * LP_H>(sm, &ok);
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(err, LP_ERR_TIMEOUT);
  } else {
    // 8 warps: warp w reads TMEM lanes 32 (w % 4).., columns 64 (w / 4)..
    const int r = (warp & 3) * 32 + lane;
    const int i = base + r;
    const int half = warp >> 2;
    float v[LP_H];
#pragma unroll
    for (int cc = 0; cc < LP_H; cc += 16)
      umma::tmem_ld16(tmem + ((uint32_t)((warp & 3) * 32) << 16) + half * LP_H + cc, v + cc);
    if (i < n) {
      float4* dst = reinterpret_cast<float4*>((half == 0 ? dh_self : dm) + (size_t)i * LP_H);
#pragma unroll
      for (int q4 = 0; q4 < LP_H / 4; q4++) dst[q4] = make_float4(v[4 * q4], v[4 * q4 + 1], v[4 * q4 + 2], v[4 * q4 + 3]);
    }
  }
  lp_end(tmem, 2 * LP_H);
}

// Transpose of the gather: dh_j = dh_self_j + sum_{i in N(j)} g_ij (dm_i / deg_i)
// with g_ij the gate seen from i (normal flipped); partials of dWe and dce.
constexpr int LP_GB_LEN = LP_H * LP_NE + LP_H;
__global__ void __launch_bounds__(256) k_lp_gather_bwd(int n, const int* __restrict__ nptr,
                                                       const int* __restrict__ nnbr, const float4* __restrict__ ef,
                                                       const float* __restrict__ invdeg,
                                                       const __nv_bfloat16* __restrict__ h_in,
                                                       const float* __restrict__ wl, const float* __restrict__ dh_self,
                                                       const float* __restrict__ dm, float* __restrict__ dh_next,
                                                       float* __restrict__ part) {
  __shared__ float red[8 * LP_GB_LEN];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, c = 2 * lane;
  const Gate2 g = load_gate(wl, c);
  float gw0[4] = {0, 0, 0, 0}, gw1[4] = {0, 0, 0, 0}, gc0 = 0.f, gc1 = 0.f;
  const int nwarps = gridDim.x * (blockDim.x >> 5);
  for (int j = blockIdx.x * (blockDim.x >> 5) + warp; j < n; j += nwarps) {
    float2 acc = *reinterpret_cast<const float2*>(&dh_self[(size_t)j * LP_H + c]);
    const float2 hj = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&h_in[(size_t)j * LP_H + c]));
    for (int p = nptr[j]; p < nptr[j + 1]; p++) {
      const int i = nnbr[p];
      const float4 e = ef[p];
      const float id = invdeg[i];
      const float2 d = *reinterpret_cast<const float2*>(&dm[(size_t)i * LP_H + c]);
      const float d0 = d.x * id, d1 = d.y * id;
      const float2 gv = gate_eval(g, e, -1.f);
      acc.x = fmaf(gv.x, d0, acc.x);
      acc.y = fmaf(gv.y, d1, acc.y);
      const float dg0 = d0 * hj.x, dg1 = d1 * hj.y;
      gc0 += dg0;
      gc1 += dg1;
      gw0[0] -= dg0 * e.x; gw0[1] -= dg0 * e.y; gw0[2] -= dg0 * e.z; gw0[3] += dg0 * e.w;
      gw1[0] -= dg1 * e.x; gw1[1] -= dg1 * e.y; gw1[2] -= dg1 * e.z; gw1[3] += dg1 * e.w;
    }
    *reinterpret_cast<float2*>(&dh_next[(size_t)j * LP_H + c]) = acc;
  }
  float* my = red + warp * LP_GB_LEN;
#pragma unroll
  for (int k = 0; k < 4; k++) {
    my[c * LP_NE + k] = gw0[k];
    my[(c + 1) * LP_NE + k] = gw1[k];
  }
  my[LP_H * LP_NE + c] = gc0;
  my[LP_H * LP_NE + c + 1] = gc1;
  lp_block_sum(red, LP_GB_LEN, part + (size_t)blockIdx.x * LP_GB_LEN);
}

// Weight gradients of one layer on the FP32 pipes: dWs = dz^T h, dWm = dz^T m,
// db = sum dz.  A block takes a run of nodes in chunks of 32; thread t owns
// row c = t / 4 and the 32 columns t % 4 + 4 k of [h | m] (interleaved, so
// the four column groups of a warp fall in different shared-memory banks).
constexpr int LP_WG_LEN = LP_H * 2 * LP_H + LP_H;
constexpr int LP_WG_CHUNK = 32;
__global__ void __launch_bounds__(256) k_lp_wgrad(int n, int nodes_per_block, const __nv_bfloat16* __restrict__ dz,
                                                  const __nv_bfloat16* __restrict__ h,
                                                  const __nv_bfloat16* __restrict__ m, float* __restrict__ part) {
  __shared__ float sdz[LP_WG_CHUNK][LP_H];
  __shared__ float shm[LP_WG_CHUNK][2 * LP_H];
  const int t = threadIdx.x;
  const int c = t >> 2, k0 = t & 3;
  float acc[32];
#pragma unroll
  for (int k = 0; k < 32; k++) acc[k] = 0.f;
  float accb = 0.f;
  const int n0 = blockIdx.x * nodes_per_block;
  const int n1 = min(n, n0 + nodes_per_block);
  for (int cb = n0; cb < n1; cb += LP_WG_CHUNK) {
    __syncthreads();
    for (int e = t; e < LP_WG_CHUNK * LP_H; e += blockDim.x) {
      const int r = e / LP_H, k = e % LP_H, i = cb + r;
      const bool in = i < n1;
      sdz[r][k] = in ? __bfloat162float(dz[(size_t)i * LP_H + k]) : 0.f;
      shm[r][k] = in ? __bfloat162float(h[(size_t)i * LP_H + k]) : 0.f;
      shm[r][LP_H + k] = in ? __bfloat162float(m[(size_t)i * LP_H + k]) : 0.f;
    }
    __syncthreads();
    for (int r = 0; r < LP_WG_CHUNK; r++) {
      const float d = sdz[r][c];
      accb += d;
#pragma unroll
      for (int k = 0; k < 32; k++) acc[k] = fmaf(d, shm[r][k0 + 4 * k], acc[k]);
    }
  }
  float* out = part + (size_t)blockIdx.x * LP_WG_LEN;
  // [Ws | Wm] rows: Ws[c][k] for k < 64, Wm[c][k - 64] for k >= 64
#pragma unroll
  for (int k = 0; k < 32; k++) {
    const int kk = k0 + 4 * k;
    if (kk < LP_H) out[c * LP_H + kk] = acc[k];
    else out[LP_H * LP_H + c * LP_H + (kk - LP_H)] = acc[k];
  }
  if (k0 == 0) out[2 * LP_H * LP_H + c] = accb;
}

// Encoder backward: dz0 = dh0 (h0 > 0); dWin = dz0^T x, dbin = sum dz0.
// Thread t owns channel c = t / 4 and inputs 3 (t % 4) .. 3 (t % 4) + 2
// (input 11 is the bias).
constexpr int LP_EB_LEN = LP_H * LP_NIN + LP_H;
__global__ void __launch_bounds__(256) k_lp_enc_bwd(int n, int nodes_per_block, const float* __restrict__ dh,
                                                    const __nv_bfloat16* __restrict__ h0, const float* __restrict__ x,
                                                    float* __restrict__ part) {
  const int t = threadIdx.x;
  const int c = t >> 2, k0 = (t & 3) * 3;
  float acc[3] = {0.f, 0.f, 0.f};
  const int n0 = blockIdx.x * nodes_per_block;
  const int n1 = min(n, n0 + nodes_per_block);
  for (int i = n0; i < n1; i++) {
    const float hv = __bfloat162float(h0[(size_t)i * LP_H + c]);
    const float d = hv > 0.f ? dh[(size_t)i * LP_H + c] : 0.f;
#pragma unroll
    for (int k = 0; k < 3; k++) {
      const int kk = k0 + k;
      acc[k] = fmaf(d, kk < LP_NIN ? x[(size_t)i * LP_NIN + kk] : 1.f, acc[k]);
    }
  }
  float* out = part + (size_t)blockIdx.x * LP_EB_LEN;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int kk = k0 + k;
    if (kk < LP_NIN) out[c * LP_NIN + kk] = acc[k];
    else out[LP_H * LP_NIN + c] = acc[k];
  }
}

// ---------------------------------------------------------------------------
// parameters
// ---------------------------------------------------------------------------

// BF16 weight images for the tensor cores, per layer: forward [Ws | Wm] as a
// 64 x 128 K-major tile, backward [Ws | Wm]^T as a 128 x 64 K-major tile.
__global__ void k_lp_pack(const float* __restrict__ w, __nv_bfloat16* __restrict__ fwd,
                          __nv_bfloat16* __restrict__ bwd) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= LP_NL * LP_IMG) return;
  const int l = t / LP_IMG, e = t % LP_IMG;
  const float* wl = w + LP_OFF_L0 + l * LP_L_SIZE;
  {
    const int r = e / (2 * LP_H), k = e % (2 * LP_H);
    const float v = k < LP_H ? wl[LP_L_WS + r * LP_H + k] : wl[LP_L_WM + r * LP_H + (k - LP_H)];
    *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<unsigned char*>(fwd + (size_t)l * LP_IMG) +
                                      umma::tile_offset(r, k, 2 * LP_H)) = __float2bfloat16(v);
  }
  {
    const int r = e / LP_H, k = e % LP_H;  // row r of [Ws | Wm]^T, column k = output channel
    const float v = r < LP_H ? wl[LP_L_WS + k * LP_H + r] : wl[LP_L_WM + k * LP_H + (r - LP_H)];
    *reinterpret_cast<__nv_bfloat16*>(reinterpret_cast<unsigned char*>(bwd + (size_t)l * LP_IMG) +
                                      umma::tile_offset(r, k, LP_H)) = __float2bfloat16(v);
  }
}

__global__ void k_lp_adam(int np, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m1,
                          float* __restrict__ m2, float lr, float b1, float b2, float eps, float bc1, float bc2) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np) return;
  const float gk = g[k];
  const float a = b1 * m1[k] + (1.f - b1) * gk;
  const float b = b2 * m2[k] + (1.f - b2) * gk * gk;
  m1[k] = a;
  m2[k] = b;
  w[k] -= lr * (a / bc1) / (sqrtf(b / bc2) + eps);
}

// oriented edge features and 1/deg of every node
__global__ void k_lp_graph(int n, const int* __restrict__ nptr, const int* __restrict__ nedg,
                           const int2* __restrict__ en, const D4* __restrict__ ea, const double* __restrict__ xyz,
                           double lmean, float4* __restrict__ ef, float* __restrict__ invdeg) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int p0 = nptr[i], p1 = nptr[i + 1];
  invdeg[i] = p1 > p0 ? 1.0f / (float)(p1 - p0) : 0.f;
  for (int p = p0; p < p1; p++) {
    const int se = nedg[p];
    const int e = se < 0 ? ~se : se;
    const float sg = se < 0 ? 1.f : -1.f;  // ~e marks the edge's first node
    const int2 nd = en[e];
    const double dx = xyz[3 * nd.y] - xyz[3 * nd.x], dy = xyz[3 * nd.y + 1] - xyz[3 * nd.x + 1],
                 dz = xyz[3 * nd.y + 2] - xyz[3 * nd.x + 2];
    const D4 a = ea[e];
    ef[p] = make_float4(sg * (float)a.x, sg * (float)a.y, sg * (float)a.z,
                        (float)(sqrt(dx * dx + dy * dy + dz * dz) / lmean));
  }
}

// t = (dq - y) / sigma in FP32 (training target)
__global__ void k_lp_target(long long n5, const double* __restrict__ dq, const double* __restrict__ y,
                            const double* __restrict__ sigma_dev, float* __restrict__ t) {
  const double sg = *sigma_dev;
  const double is = sg > 0.0 ? 1.0 / sg : 0.0;
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n5; k += (long long)gridDim.x * blockDim.x)
    t[k] = (float)((dq[k] - y[k]) * is);
}
