// binary32 Stockham group kernel for sm_103a (the FP32 variant of the path).
//
// Same structure as the binary64 group kernel (stockham_f64.cu): one CTA loads a tile of
// sub-problems into shared memory, runs every pass of its group there, stores the tile.
// The butterflies are the same generated operation DAGs evaluated in binary32; twiddle tables
// are the binary64 exact-integer tables rounded to binary32, and the passes the planner marks
// (the last passes of sizes >= 2^16) multiply by twiddles held as binary32 (hi, lo) pairs with
// compensated products, which removes the twiddle-rounding error from those passes.  At 8
// bytes per point and 37 T binary32 instructions/s this variant is bound by HBM, not by the
// arithmetic.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "stockham_dev.cuh"

namespace lfg {
using namespace dev;
namespace {

template <bool FWD>
__global__ void __launch_bounds__(kGroupThreads)
group_kernel_f32(const GroupDesc g, const float2* in, float2* out) {
  extern __shared__ float2 smem_f32[];
  const int64_t s0 = (int64_t)blockIdx.x * g.C;
  const int64_t rem = g.total_sub - s0;
  const int C = rem < g.C ? (int)rem : g.C;
  process_tile<float, FWD>(g, StridedLines{g.in_line, g.out_line}, s0, C, in, out, smem_f32);
}

// ---- bulk-async (TMA) staging ------------------------------------------------------------

constexpr int kStages = 2;                 // tiles in flight per CTA besides the one computed
constexpr uint32_t kSpinLimit = 1u << 22;  // bounded mbarrier polls (each poll may suspend)

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

// One contiguous global -> shared copy by the bulk-copy (TMA) engine, completing on `bar`.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_test(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
  return ok != 0;
}

// Poll at most `limit` times; false if the phase did not complete in time.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit = kSpinLimit) {
  for (uint32_t i = 0; i < limit; ++i)
    if (mbar_test(bar, parity)) return true;
  return false;
}

// ---- pass policies of the persistent kernel ------------------------------------------------

// Any plan: the runtime pass descriptors of the group (stockham_dev.cuh).  Pass 0 reads the
// unpadded stage buffer a bulk copy filled.
struct GenericPasses {
  template <bool FWD>
  static __device__ __forceinline__ void pass(int t, const float2* src, float2* dst, int C,
                                              const GroupDesc& g) {
    if (t == 0) run_pass_t<float, FWD, false>(src, dst, C, g.M, g.pass[t], -1, g.nsub, g.fd_nsub);
    else run_pass_t<float, FWD>(src, dst, C, g.M, g.pass[t], -1, g.nsub, g.fd_nsub);
  }
};

// One pass of a one-group power-of-two plan with compile-time geometry: sub-problems of M
// points, radix R, NS = product of the earlier radices (also the twiddle rows' length, a
// single group's table index being k).  The same codelet on the same operands as the generic
// pass, so the same bits; what the constants remove is index arithmetic: divisions by M/R and
// NS become shifts and masks, and the padded shared-memory addresses of a butterfly's inputs
// and outputs become one base plus immediate offsets wherever the stride in r is a multiple
// of 16 (spad(x + 16 m) = spad(x) + 17 m).
template <bool FWD, int M, int R, int NS, bool SRCPAD>
__device__ __forceinline__ void pass_pow2(const float2* __restrict__ src, float2* __restrict__ dst,
                                          int C, const float2* __restrict__ tw) {
  constexpr int MR = M / R;
  constexpr int PM = sub_pitch(M);
  constexpr bool TW = NS > 1;
  static_assert((M & (M - 1)) == 0 && (R & (R - 1)) == 0 && M % R == 0, "power-of-two pass");
  const int nb = C * MR;
  const float one = 1.0f, nz = -0.0f;   // (the binary32 codelets do not use them)
  for (int q = threadIdx.x; q < nb; q += blockDim.x) {
    const int c = q / MR;
    const int j = q % MR;
    float x[TW ? 4 * R - 2 : 2 * R];
    float y[2 * R];
    const float2* sc = src + c * (SRCPAD ? PM : M);
    if (SRCPAD && MR % 16 == 0) {
      const float2* s0 = sc + spad(j);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float2 v = s0[r * (MR + MR / 16)];
        x[2 * r] = v.x;
        x[2 * r + 1] = v.y;
      }
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int si = j + r * MR;
        const float2 v = sc[SRCPAD ? spad(si) : si];
        x[2 * r] = v.x;
        x[2 * r + 1] = v.y;
      }
    }
    const int b = j / NS;
    const int k = j % NS;
    if (TW) {
      const float2* __restrict__ w = tw + k;
#pragma unroll
      for (int r = 0; r < R - 1; ++r) {
        const float2 v = __ldg(w + r * NS);
        x[2 * R + 2 * r] = v.x;
        x[2 * R + 2 * r + 1] = v.y;
      }
    }
    BflyF<FWD, R, TW>::run(x, y, one, nz);
    const int d0 = b * NS * R + k;
    float2* dc = dst + c * PM;
    if (NS % 16 == 0) {
      float2* o = dc + spad(d0);
#pragma unroll
      for (int r = 0; r < R; ++r) o[r * (NS + NS / 16)] = make_float2(y[2 * r], y[2 * r + 1]);
    } else if (NS == 1 && R == 16) {
      float2* o = dc + 17 * b;   // outputs 16 b .. 16 b + 15: spad(16 b + r) = 17 b + r
#pragma unroll
      for (int r = 0; r < R; ++r) o[r] = make_float2(y[2 * r], y[2 * r + 1]);
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) dc[spad(d0 + r * NS)] = make_float2(y[2 * r], y[2 * r + 1]);
    }
  }
}

// A one-group power-of-two plan with radices R0, R1, R2, R3 (0: no such pass), M points.
template <int M, int R0, int R1, int R2, int R3>
struct Pow2Passes {
  template <bool FWD>
  static __device__ __forceinline__ void pass(int t, const float2* src, float2* dst, int C,
                                              const GroupDesc& g) {
    switch (t) {
      case 0:
        pass_pow2<FWD, M, R0, 1, false>(src, dst, C, nullptr);
        break;
      case 1:
        if constexpr (R1 > 0)
          pass_pow2<FWD, M, R1, R0, true>(src, dst, C, static_cast<const float2*>(g.pass[1].tw));
        break;
      case 2:
        if constexpr (R2 > 0)
          pass_pow2<FWD, M, R2, R0 * R1, true>(src, dst, C, static_cast<const float2*>(g.pass[2].tw));
        break;
      default:
        if constexpr (R3 > 0)
          pass_pow2<FWD, M, R3, R0 * R1 * R2, true>(src, dst, C, static_cast<const float2*>(g.pass[3].tw));
        break;
    }
  }
};

// Persistent binary32 kernel for back-to-back lines of one pass group: each CTA walks the
// tiles t = blockIdx.x, blockIdx.x + gridDim.x, ...; the bulk-copy engine prefetches kStages
// tiles ahead into stage buffers (one mbarrier each) while the CTA runs the passes of the
// current tile in two work buffers, so HBM reads overlap the arithmetic.  The first pass
// reads the stage buffer directly, after which the buffer is refilled with a later tile.
// A wait that gives up sets *status = 1, waits (bounded) for this CTA's copies in flight and
// returns.  tile_limit bounds the tile waits (kSpinLimit; 0 in tests of the give-up path, whose
// drain still uses kSpinLimit).
template <bool FWD, class Passes = GenericPasses>
__global__ void __launch_bounds__(kGroupThreads, 3)
stream_kernel_f32(const GroupDesc g, const float2* __restrict__ in, float2* __restrict__ out,
                  int64_t lines, int* status, uint32_t tile_limit) {
  extern __shared__ __align__(128) float2 smem_f32s[];
  __shared__ __align__(8) uint64_t bars[kStages];
  const int M = g.M, CM = g.C * g.M, PM = sub_pitch(g.M);
  float2* A = smem_f32s + kStages * CM;       // stage buffers unpadded (bulk-copy targets)
  float2* B = A + tile_elems(g.C, M);
  const int64_t ntiles = (lines + g.C - 1) / g.C;
  bool pending[kStages];
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  auto issue = [&](int s, int64_t tile) {   // thread 0 only
    const int64_t l0 = tile * g.C;
    const int cnt = (int)min((int64_t)g.C, lines - l0);
    const uint32_t bytes = (uint32_t)cnt * M * sizeof(float2);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&bars[s], bytes);
    bulk_load(smem_f32s + s * CM, in + l0 * M, bytes, &bars[s]);
  };
  for (int s = 0; s < kStages; ++s) {
    const int64_t t = blockIdx.x + (int64_t)s * gridDim.x;
    pending[s] = t < ntiles;
    if (threadIdx.x == 0 && pending[s]) issue(s, t);
  }
  uint32_t parity = 0;   // bit s: parity of stage s's next phase
  int s = 0;
  bool failed = false;
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t l0 = tile * g.C;
    const int C = (int)min((int64_t)g.C, lines - l0);
    const bool ok = __syncthreads_and(mbar_wait(&bars[s], (parity >> s) & 1, tile_limit));
    if (!ok) {
      failed = true;
      break;
    }
    parity ^= 1u << s;
    pending[s] = false;
    float2* src = smem_f32s + s * CM;
    float2* dst = A;
    for (int t = 0; t < g.npass; ++t) {
      Passes::template pass<FWD>(t, src, dst, C, g);
      __syncthreads();
      if (t == 0) {
        // the stage buffer has been read: refill it with this CTA's tile kStages ahead
        const int64_t next = tile + (int64_t)kStages * gridDim.x;
        pending[s] = next < ntiles;
        if (threadIdx.x == 0 && pending[s]) issue(s, next);
        src = A;
        dst = B;
      } else {
        float2* tmp = src;
        src = dst;
        dst = tmp;
      }
    }
    // store the tile (contiguous): two complex values per 16-byte store
    float4* o4 = reinterpret_cast<float4*>(out + l0 * M);
    const int n4 = C * M / 2;
    const float sc = g.scale_f32;
    const bool flat = (M & 15) == 0;   // then c * PM + spad(ii) = spad(c * M + ii)
    for (int i = threadIdx.x; i < n4; i += blockDim.x) {
      const int e = 2 * i;
      int t0, t1;
      if (flat) {
        t0 = spad(e);
        t1 = spad(e + 1);
      } else {
        const int c = fdiv(e, g.fd_m), ii = e - c * M;   // M even: ii + 1 < M
        t0 = c * PM + spad(ii);
        t1 = c * PM + spad(ii + 1);
      }
      const float2 a = src[t0], b = src[t1];
      if (g.unit_scale) o4[i] = make_float4(a.x, a.y, b.x, b.y);
      else o4[i] = make_float4(__fmul_rn(a.x, sc), __fmul_rn(a.y, sc), __fmul_rn(b.x, sc), __fmul_rn(b.y, sc));
    }
    __syncthreads();
    s = (s + 1) % kStages;
  }
  if (failed) {
    if (threadIdx.x == 0) atomicExch(status, 1);
    // let this CTA's own copies in flight land before the CTA (and its smem) goes away
    for (int k = 0; k < kStages; ++k)
      if (pending[k]) mbar_wait(&bars[k], (parity >> k) & 1);
  }
}

// ---- asynchronous element copies (cp.async) for strided tiles ------------------------------

__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem_addr(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Issue the copies of tile `s0` (C of g.C sub-problems) into the padded tile buffer S; same
// element order and addressing as the synchronous tile load (stockham_dev.cuh: copy_tile).
__device__ __forceinline__ void load_tile_async(float2* S, const float2* in, const GroupDesc& g,
                                                int64_t s0, int C) {
  // descriptor fields in registers (each cp.async is a compiler memory barrier)
  const int M = g.M, nsub = g.nsub, PM = sub_pitch(M), gC = g.C;
  const int64_t in_line = g.in_line, in_sub = g.in_sub, in_elem = g.in_elem;
  const FastDiv fd_m = g.fd_m, fd_c = g.fd_c, fd_nsub = g.fd_nsub;
  const int64_t line0 = s0 / nsub;
  const int sub0 = (int)(s0 - line0 * nsub);
  const bool elem_fast = in_elem == 1;
  const int nn = elem_fast ? C * M : gC * M;
#pragma unroll 4
  for (int idx = threadIdx.x; idx < nn; idx += blockDim.x) {
    int c, i;
    if (elem_fast) {
      c = fdiv(idx, fd_m);
      i = idx - c * M;
    } else {
      i = fdiv(idx, fd_c);
      c = idx - i * gC;
      if (c >= C) continue;
    }
    const int t = sub0 + c;
    const int ql = fdiv(t, fd_nsub);
    const int64_t a = (line0 + ql) * in_line + (int64_t)(t - ql * nsub) * in_sub +
                      (int64_t)i * in_elem;
    cp_async8(S + c * PM + spad(i), in + a);
  }
  cp_async_commit();
}

// ---- tile policies of the strided-tile kernel ----------------------------------------------

// Any group: runtime pass descriptors, the padded tile layout of stockham_dev.cuh.
struct GenericTiles {
  static __device__ __forceinline__ int pitch(const GroupDesc& g) { return sub_pitch(g.M); }
  static __device__ __forceinline__ void load(float2* S, const float2* in, const GroupDesc& g,
                                              int64_t s0, int C) {
    load_tile_async(S, in, g, s0, C);
  }
  template <bool FWD>
  static __device__ __forceinline__ void pass(int t, const float2* src, float2* dst, int C,
                                              const GroupDesc& g, int sub0) {
    run_pass_t<float, FWD>(src, dst, C, g.M, g.pass[t], sub0, g.nsub, g.fd_nsub);
  }
  static __device__ __forceinline__ void store(const float2* src, float2* out, const GroupDesc& g,
                                               int64_t s0, int C) {
    copy_tile<float, false>(const_cast<float2*>(src), nullptr, out, g,
                            StridedLines{g.in_line, g.out_line}, s0, C);
  }
};

// One pass of a group of a two-group power-of-two plan, compile-time geometry: sub-problems of
// M points at pitch PM, radix R, NSL = product of the group's earlier radices; TWSUB: a second
// group, whose table index is m * NSL + k with m = (sub0 + c) mod NSUB (rows of NSUB * NSL);
// MODE 0 untwiddled, 1 twiddled, 2 compensated (hi, lo) twiddles -- the same operations on the
// same operands as pass_t (stockham_dev.cuh), so the same bits.
template <bool FWD, int M, int PM, int R, int NSL, int NSUB, bool TWSUB, int MODE>
__device__ __forceinline__ void pass_group_pow2(const float2* __restrict__ src,
                                                float2* __restrict__ dst, int C,
                                                const float2* __restrict__ tw, int sub0) {
  using P = Prec<float>;
  constexpr int MR = M / R;
  constexpr int NSG = TWSUB ? NSUB * NSL : NSL;
  constexpr bool TW = MODE == 1;
  static_assert((M & (M - 1)) == 0 && (R & (R - 1)) == 0 && (NSUB & (NSUB - 1)) == 0, "powers of two");
  const int nb = C * MR;
  const float one = 1.0f, nz = -0.0f;   // (the binary32 codelets do not use them)
  for (int q = threadIdx.x; q < nb; q += blockDim.x) {
    const int c = q / MR;
    const int j = q % MR;
    float x[TW ? 4 * R - 2 : 2 * R];
    float y[2 * R];
    const float2* sc = src + c * PM;
    if (MR % 16 == 0) {
      const float2* s0 = sc + spad(j);
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float2 v = s0[r * (MR + MR / 16)];
        x[2 * r] = v.x;
        x[2 * r + 1] = v.y;
      }
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const float2 v = sc[spad(j + r * MR)];
        x[2 * r] = v.x;
        x[2 * r + 1] = v.y;
      }
    }
    const int b = j / NSL;
    const int k = j % NSL;
    const int kg = TWSUB ? ((sub0 + c) % NSUB) * NSL + k : k;
    if (MODE == 1) {
      const float2* __restrict__ w = tw + kg;
#pragma unroll
      for (int r = 0; r < R - 1; ++r) {
        const float2 v = __ldg(w + r * NSG);
        x[2 * R + 2 * r] = v.x;
        x[2 * R + 2 * r + 1] = v.y;
      }
    } else if (MODE == 2) {
      const float2* __restrict__ wh = tw + kg;
      const float2* __restrict__ wl = wh + (R - 1) * NSG;
#pragma unroll
      for (int r = 1; r < R; ++r) {
        const float2 h = __ldg(wh + (r - 1) * NSG), l = __ldg(wl + (r - 1) * NSG);
        const float wrh = h.x, wih = h.y, wrl = l.x, wil = l.y;
        const float a = x[2 * r], bi = x[2 * r + 1];
        const float cr = P::fma(a, wrl, -P::mul(bi, wil));
        const float ci = P::fma(a, wil, P::mul(bi, wrl));
        x[2 * r] = P::fma(a, wrh, P::fma(-bi, wih, cr));
        x[2 * r + 1] = P::fma(a, wih, P::fma(bi, wrh, ci));
      }
    }
    BflyF<FWD, R, TW>::run(x, y, one, nz);
    const int d0 = b * NSL * R + k;
    float2* dc = dst + c * PM;
    if (NSL % 16 == 0) {
      float2* o = dc + spad(d0);
#pragma unroll
      for (int r = 0; r < R; ++r) o[r * (NSL + NSL / 16)] = make_float2(y[2 * r], y[2 * r + 1]);
    } else if (NSL == 1 && R == 16) {
      float2* o = dc + 17 * b;
#pragma unroll
      for (int r = 0; r < R; ++r) o[r] = make_float2(y[2 * r], y[2 * r + 1]);
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) dc[spad(d0 + r * NSL)] = make_float2(y[2 * r], y[2 * r + 1]);
    }
  }
}

// A group of a two-group power-of-two plan with radices R0, R1, R2 (0: no such pass), M
// points per sub-problem, the other group's size NSUB (a second group: TWSUB, its twiddles
// compensated when COMP).  Tiles use an odd pitch, so the strided copies, whose neighbouring
// threads take neighbouring sub-problems, spread over the banks; the copies walk their
// elements with running indices.
template <int M, int NSUB, bool TWSUB, bool COMP, int R0, int R1, int R2>
struct Pow2GroupTiles {
  static constexpr int PM = sub_pitch(M) | 1;
  static constexpr int MODE_T = TWSUB ? (COMP ? 2 : 1) : 1;   // twiddled passes
  static __device__ __forceinline__ int pitch(const GroupDesc&) { return PM; }
  static __device__ __forceinline__ void load(float2* S, const float2* in, const GroupDesc& g,
                                              int64_t s0, int C) {
    // element (c, i): neighbouring threads take neighbouring sub-problems (runs of C)
    const int gC = g.C, nsub = g.nsub;
    const FastDiv fd_c = g.fd_c, fd_nsub = g.fd_nsub;
    const int64_t in_line = g.in_line, in_sub = g.in_sub, in_elem = g.in_elem;
    const int64_t line0 = s0 / nsub;
    const int sub_0 = (int)(s0 - line0 * nsub);
    const bool one_line = sub_0 + C <= nsub;
    const float2* base = in + line0 * in_line + (int64_t)sub_0 * in_sub;
    const int S_ = blockDim.x;
    int i = fdiv(threadIdx.x, fd_c);
    int c = (int)threadIdx.x - i * gC;
    const int di = fdiv(S_, fd_c), dc = S_ - di * gC;
    for (int idx = threadIdx.x; idx < gC * M; idx += S_) {
      if (c < C) {
        const float2* a;
        if (one_line) {
          a = base + (int64_t)c * in_sub + (int64_t)i * in_elem;
        } else {
          const int t = sub_0 + c;
          const int ql = fdiv(t, fd_nsub);
          a = in + (line0 + ql) * in_line + (int64_t)(t - ql * nsub) * in_sub + (int64_t)i * in_elem;
        }
        cp_async8(S + c * PM + spad(i), a);
      }
      c += dc;
      i += di;
      if (c >= gC) {
        c -= gC;
        ++i;
      }
    }
    cp_async_commit();
  }
  template <bool FWD>
  static __device__ __forceinline__ void pass(int t, const float2* src, float2* dst, int C,
                                              const GroupDesc& g, int sub0) {
    const float2* tw = static_cast<const float2*>(g.pass[t].tw);
    switch (t) {
      case 0:
        pass_group_pow2<FWD, M, PM, R0, 1, NSUB, TWSUB, TWSUB ? MODE_T : 0>(src, dst, C, tw, sub0);
        break;
      case 1:
        if constexpr (R1 > 0)
          pass_group_pow2<FWD, M, PM, R1, R0, NSUB, TWSUB, MODE_T>(src, dst, C, tw, sub0);
        break;
      default:
        if constexpr (R2 > 0)
          pass_group_pow2<FWD, M, PM, R2, R0 * R1, NSUB, TWSUB, MODE_T>(src, dst, C, tw, sub0);
        break;
    }
  }
  static __device__ __forceinline__ void store(const float2* src, float2* out, const GroupDesc& g,
                                               int64_t s0, int C) {
    const int gC = g.C, nsub = g.nsub;
    const FastDiv fd_c = g.fd_c, fd_nsub = g.fd_nsub;
    const int64_t out_line = g.out_line, out_sub = g.out_sub, out_elem = g.out_elem;
    const int64_t line0 = s0 / nsub;
    const int sub_0 = (int)(s0 - line0 * nsub);
    const bool unit = g.unit_scale != 0;
    const float sc = g.scale_f32;
    const int S_ = blockDim.x;
    if (out_elem == 1) {
      // contiguous sub-problems: element (c, i), neighbouring threads along i
      int c = (int)threadIdx.x / M;
      int i = (int)threadIdx.x - c * M;
      const int dc = S_ / M, di = S_ - dc * M;
      for (int idx = threadIdx.x; idx < C * M; idx += S_) {
        const int t = sub_0 + c;
        const int ql = fdiv(t, fd_nsub);
        const int64_t a = (line0 + ql) * out_line + (int64_t)(t - ql * nsub) * out_sub + i;
        const float2 v = src[c * PM + spad(i)];
        out[a] = unit ? v : make_float2(__fmul_rn(v.x, sc), __fmul_rn(v.y, sc));
        c += dc;
        i += di;
        if (i >= M) {
          i -= M;
          ++c;
        }
      }
      return;
    }
    int i = fdiv(threadIdx.x, fd_c);
    int c = (int)threadIdx.x - i * gC;
    const int di = fdiv(S_, fd_c), dc = S_ - di * gC;
    for (int idx = threadIdx.x; idx < gC * M; idx += S_) {
      if (c < C) {
        const int t = sub_0 + c;
        const int ql = fdiv(t, fd_nsub);
        const int64_t a = (line0 + ql) * out_line + (int64_t)(t - ql * nsub) * out_sub + (int64_t)i * out_elem;
        const float2 v = src[c * PM + spad(i)];
        out[a] = unit ? v : make_float2(__fmul_rn(v.x, sc), __fmul_rn(v.y, sc));
      }
      c += dc;
      i += di;
      if (c >= gC) {
        c -= gC;
        ++i;
      }
    }
  }
};

// Persistent binary32 kernel for tiles of strided sub-problems (the groups of two-group plans
// and strided batches): each CTA walks the tiles blockIdx.x, blockIdx.x + gridDim.x, ...;
// the next tile's elements are copied asynchronously into a stage buffer while the CTA runs
// the later passes of the current tile and stores it, so HBM reads overlap the arithmetic
// and the stores.  Waits are cp.async group waits (no polling).
template <bool FWD, class Tiles = GenericTiles>
__global__ void __launch_bounds__(kGroupThreads)
tile_stream_kernel_f32(const GroupDesc g, const float2* in, float2* out) {
  extern __shared__ __align__(16) float2 smem_ts[];
  const int PE = g.C * Tiles::pitch(g);
  float2* S = smem_ts;
  float2* A = S + PE;
  float2* B = A + PE;
  const int64_t ntiles = (g.total_sub + g.C - 1) / g.C;
  auto count = [&](int64_t tile) { return (int)min((int64_t)g.C, g.total_sub - tile * g.C); };
  if ((int64_t)blockIdx.x < ntiles) Tiles::load(S, in, g, (int64_t)blockIdx.x * g.C, count(blockIdx.x));
  for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int64_t s0 = tile * g.C;
    const int C = count(tile);
    cp_async_wait_all();
    __syncthreads();
    const int sub0 = g.twsub ? (int)(s0 % g.nsub) : -1;
    Tiles::template pass<FWD>(0, S, A, C, g, sub0);
    __syncthreads();
    // the stage buffer has been consumed: start copying this CTA's next tile
    const int64_t next = tile + gridDim.x;
    if (next < ntiles) Tiles::load(S, in, g, next * g.C, count(next));
    float2* src = A;
    float2* dst = B;
    for (int t = 1; t < g.npass; ++t) {
      Tiles::template pass<FWD>(t, src, dst, C, g, sub0);
      __syncthreads();
      float2* tmp = src;
      src = dst;
      dst = tmp;
    }
    Tiles::store(src, out, g, s0, C);
  }
  cp_async_wait_all();
}

template <class K>
cudaError_t allow_max_smem(K kern) {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, kern);
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)(kMaxSmemBytes - a.sharedSizeBytes));
}

using StreamFn = void (*)(const GroupDesc, const float2*, float2*, int64_t, int*, uint32_t);

// The persistent kernel of plan variant v: -1 = any plan (runtime pass descriptors), else the
// power-of-two plan kPow2Plans[v] with compile-time passes.
template <bool FWD>
StreamFn stream_fn(int v) {
  switch (v) {
    case 0: return stream_kernel_f32<FWD, Pow2Passes<16, 16, 0, 0, 0>>;
    case 1: return stream_kernel_f32<FWD, Pow2Passes<32, 16, 2, 0, 0>>;
    case 2: return stream_kernel_f32<FWD, Pow2Passes<64, 16, 4, 0, 0>>;
    case 3: return stream_kernel_f32<FWD, Pow2Passes<128, 16, 8, 0, 0>>;
    case 4: return stream_kernel_f32<FWD, Pow2Passes<256, 16, 16, 0, 0>>;
    case 5: return stream_kernel_f32<FWD, Pow2Passes<512, 16, 16, 2, 0>>;
    case 6: return stream_kernel_f32<FWD, Pow2Passes<1024, 16, 16, 4, 0>>;
    case 7: return stream_kernel_f32<FWD, Pow2Passes<2048, 16, 16, 8, 0>>;
    case 8: return stream_kernel_f32<FWD, Pow2Passes<4096, 16, 16, 16, 0>>;
    case 9: return stream_kernel_f32<FWD, Pow2Passes<8192, 16, 16, 16, 2>>;
    default: return stream_kernel_f32<FWD, GenericPasses>;
  }
}

// The (size, radices) of the compile-time variants above, in the same order.
struct Pow2Plan {
  int n;
  int r[4];
};
constexpr Pow2Plan kPow2Plans[] = {
    {16, {16, 0, 0, 0}},    {32, {16, 2, 0, 0}},    {64, {16, 4, 0, 0}},
    {128, {16, 8, 0, 0}},   {256, {16, 16, 0, 0}},  {512, {16, 16, 2, 0}},
    {1024, {16, 16, 4, 0}}, {2048, {16, 16, 8, 0}}, {4096, {16, 16, 16, 0}},
    {8192, {16, 16, 16, 2}}};
constexpr int kPow2Variants = (int)(sizeof(kPow2Plans) / sizeof(kPow2Plans[0]));

using TileFn = void (*)(const GroupDesc, const float2*, float2*);

// The groups of the two-group power-of-two binary32 plans (2^14 .. 2^18) with compile-time
// passes: M, the other group's size (a second group's sub-problems per line), second group,
// compensated twiddles, radices.  -1 = any group (runtime descriptors).
struct TileGroup {
  int M, nsub, twsub, comp, r[3];
};
constexpr TileGroup kTileGroups[] = {
    {128, 0, 0, 0, {16, 8, 0}},    {256, 0, 0, 0, {16, 16, 0}},   {512, 0, 0, 0, {16, 16, 2}},
    {128, 128, 1, 0, {16, 8, 0}},  {128, 256, 1, 0, {16, 8, 0}},  {256, 256, 1, 0, {16, 16, 0}},
    {256, 256, 1, 1, {16, 16, 0}}, {512, 256, 1, 0, {2, 16, 16}}, {512, 256, 1, 1, {2, 16, 16}},
    {512, 512, 1, 0, {16, 16, 2}}, {512, 512, 1, 1, {16, 16, 2}}};
constexpr int kTileVariants = (int)(sizeof(kTileGroups) / sizeof(kTileGroups[0]));

template <bool FWD>
TileFn tile_fn(int v) {
  switch (v) {
    case 0: return tile_stream_kernel_f32<FWD, Pow2GroupTiles<128, 1, false, false, 16, 8, 0>>;
    case 1: return tile_stream_kernel_f32<FWD, Pow2GroupTiles<256, 1, false, false, 16, 16, 0>>;
    case 2: return tile_stream_kernel_f32<FWD, Pow2GroupTiles<512, 1, false, false, 16, 16, 2>>;
    case 3: return tile_stream_kernel_f32<FWD, Pow2GroupTiles<128, 128, true, false, 16, 8, 0>>;
    case 4: return tile_stream_kernel_f32<FWD, Pow2GroupTiles<128, 256, true, false, 16, 8, 0>>;
    case 5: return tile_stream_kernel_f32<FWD, Pow2GroupTiles<256, 256, true, false, 16, 16, 0>>;
    case 6: return tile_stream_kernel_f32<FWD, Pow2GroupTiles<256, 256, true, true, 16, 16, 0>>;
    case 7: return tile_stream_kernel_f32<FWD, Pow2GroupTiles<512, 256, true, false, 2, 16, 16>>;
    case 8: return tile_stream_kernel_f32<FWD, Pow2GroupTiles<512, 256, true, true, 2, 16, 16>>;
    case 9: return tile_stream_kernel_f32<FWD, Pow2GroupTiles<512, 512, true, false, 16, 16, 2>>;
    case 10: return tile_stream_kernel_f32<FWD, Pow2GroupTiles<512, 512, true, true, 16, 16, 2>>;
    default: return tile_stream_kernel_f32<FWD, GenericTiles>;
  }
}

// Shared memory of the strided-tile kernel: three tiles (stage and two work buffers); the
// compile-time variants use an odd pitch.
size_t tile_smem_bytes(const GroupDesc& g, int v) {
  const int pitch = v >= 0 && v < kTileVariants ? (sub_pitch(g.M) | 1) : sub_pitch(g.M);
  return 3 * (size_t)g.C * pitch * sizeof(float2);
}

}  // namespace

int tile_variant_f32(const GroupDesc& g) {
  for (int v = 0; v < kTileVariants; ++v) {
    const TileGroup& t = kTileGroups[v];
    if (t.M != g.M || t.twsub != g.twsub) continue;
    if (t.twsub && t.nsub != g.nsub) continue;
    int np = 0;
    while (np < 3 && t.r[np] > 0) ++np;
    if (np != g.npass) continue;
    bool ok = true;
    for (int p = 0; p < np && ok; ++p) {
      ok = g.pass[p].R == t.r[p] && g.pass[p].comp == (t.twsub ? t.comp : 0);
      // a first group's first pass is untwiddled, every other pass twiddled
      ok = ok && ((g.pass[p].tw == nullptr) == (!t.twsub && p == 0));
    }
    if (ok) return v;
  }
  return -1;
}

int stream_variant_f32(int64_t n, const std::vector<int>& rs) {
  for (int v = 0; v < kPow2Variants; ++v) {
    const Pow2Plan& p = kPow2Plans[v];
    if (p.n != n) continue;
    size_t np = 0;
    while (np < 4 && p.r[np] > 0) ++np;
    if (np != rs.size()) return -1;
    for (size_t t = 0; t < np; ++t)
      if (p.r[t] != rs[t]) return -1;
    return v;
  }
  return -1;
}

cudaError_t prepare_group_kernels_f32() {
  cudaError_t e = allow_max_smem(group_kernel_f32<true>);
  if (e != cudaSuccess) return e;
  if ((e = allow_max_smem(group_kernel_f32<false>)) != cudaSuccess) return e;
  for (int v = -1; v < kPow2Variants; ++v) {
    if ((e = allow_max_smem(stream_fn<true>(v))) != cudaSuccess) return e;
    if ((e = allow_max_smem(stream_fn<false>(v))) != cudaSuccess) return e;
  }
  for (int v = -1; v < kTileVariants; ++v) {
    if ((e = allow_max_smem(tile_fn<true>(v))) != cudaSuccess) return e;
    if ((e = allow_max_smem(tile_fn<false>(v))) != cudaSuccess) return e;
  }
  return prepare_direct_kernels_f32();
}

size_t tile_stream_smem_bytes_f32(const GroupDesc& g, int variant) {
  return tile_smem_bytes(g, variant);
}

int tile_stream_blocks_per_sm_f32(const GroupDesc& g, int variant) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, tile_fn<true>(variant), kGroupThreads,
                                                    tile_smem_bytes(g, variant)) != cudaSuccess)
    return 1;
  return nb > 0 ? nb : 1;
}

cudaError_t launch_tile_stream_f32(const GroupDesc& gd, bool fwd, const void* in, void* out,
                                   unsigned grid, cudaStream_t stream, int variant) {
  GroupDesc g = gd;
  set_divisors(g);
  const int64_t ntiles = (g.total_sub + g.C - 1) / g.C;
  if (ntiles <= 0) return cudaSuccess;
  if (variant >= kTileVariants) variant = -1;
  const unsigned gr = (unsigned)std::min<int64_t>(grid, ntiles);
  const TileFn kern = fwd ? tile_fn<true>(variant) : tile_fn<false>(variant);
  kern<<<gr, kGroupThreads, tile_smem_bytes(g, variant), stream>>>(
      g, static_cast<const float2*>(in), static_cast<float2*>(out));
  return cudaGetLastError();
}

size_t stream_smem_bytes_f32(const GroupDesc& g) {
  return ((size_t)kStages * g.C * g.M + 2 * (size_t)tile_elems(g.C, g.M)) * sizeof(float2);
}

int stream_blocks_per_sm_f32(const GroupDesc& g, int variant) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, stream_fn<true>(variant), kGroupThreads,
                                                    stream_smem_bytes_f32(g)) != cudaSuccess)
    return 1;
  return nb > 0 ? nb : 1;
}

cudaError_t launch_stream_f32(const GroupDesc& gd, bool fwd, const void* in, void* out,
                              int64_t lines, unsigned grid, int* status, cudaStream_t stream,
                              bool give_up, int variant) {
  GroupDesc g = gd;
  set_divisors(g);
  if (lines <= 0) return cudaSuccess;
  if (variant >= kPow2Variants) variant = -1;
  const StreamFn kern = fwd ? stream_fn<true>(variant) : stream_fn<false>(variant);
  kern<<<grid, kGroupThreads, stream_smem_bytes_f32(g), stream>>>(
      g, static_cast<const float2*>(in), static_cast<float2*>(out), lines, status,
      give_up ? 0u : kSpinLimit);
  return cudaGetLastError();
}

cudaError_t launch_group_f32(const GroupDesc& gd, bool fwd, const void* in, void* out,
                             cudaStream_t stream) {
  GroupDesc g = gd;
  set_divisors(g);
  const size_t smem = 2 * (size_t)tile_elems(g.C, g.M) * sizeof(float2);
  const int64_t grid = (g.total_sub + g.C - 1) / g.C;
  if (grid <= 0) return cudaSuccess;
  auto kern = fwd ? group_kernel_f32<true> : group_kernel_f32<false>;
  kern<<<(unsigned)grid, kGroupThreads, smem, stream>>>(g, static_cast<const float2*>(in),
                                                        static_cast<float2*>(out));
  return cudaGetLastError();
}

}  // namespace lfg
