// Device code of the tropical contraction engine (sm_103a).
//
//   leaves_tile    GenericTensorNetworks IndependentSet tensors, built on the
//                  device: vertex [0, w], edge [[0,0],[0,-inf]], sliced labels
//                  restricted to the item's values
//   stream_tile    one CTA tile of a fused contraction node: bit-permuted
//                  gathers of A and B into XOR-swizzled shared memory,
//                  max-plus reduction, coalesced store of C
//   gemm_tile      register-blocked gather GEMM tile for GEMM-shaped nodes
//   final_tile     max over the root tensor + r (warp-shuffle reduction)
//   gemm_k1        batched max-plus GEMM on canonical column-major operands,
//                  packed add.f32x2 + three-input max.f32 (the plain path)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "tb_internal.h"

namespace tb {

// ---------------------------------------------------------------------------
// semiring
// ---------------------------------------------------------------------------
// packed f32 pair add (one FADD2 for two sums) and three-input max
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ float max3(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float lo32(uint64_t x) { return __uint_as_float((uint32_t)x); }
__device__ __forceinline__ float hi32(uint64_t x) { return __uint_as_float((uint32_t)(x >> 32)); }
__device__ __forceinline__ uint64_t pack2(float x, float y) {
  return (uint64_t)__float_as_uint(x) | ((uint64_t)__float_as_uint(y) << 32);
}

template <typename T>
struct Trop;

template <>
struct Trop<float> {
  static __device__ __forceinline__ float neg() { return __int_as_float(0xff800000); }
  static __device__ __forceinline__ float mac(float acc, float a, float b) { return fmaxf(acc, a + b); }
  // two terms: max(acc, a0 + b0, a1 + b1) as one packed add and one 3-input max
  static __device__ __forceinline__ float mac2(float acc, float a0, float a1, float b0, float b1) {
    const uint64_t s = add2(pack2(a0, a1), pack2(b0, b1));
    return max3(acc, lo32(s), hi32(s));
  }
  static __device__ __forceinline__ float mx(float a, float b) { return fmaxf(a, b); }
  static __device__ __forceinline__ float from_w(float w) { return w; }
  static __device__ __forceinline__ float to_f(float v) { return v; }
};

template <>
struct Trop<int32_t> {
  static __device__ __forceinline__ int32_t neg() { return -536870912; }
  // DPX: max(a + b, acc) in one instruction
  static __device__ __forceinline__ int32_t mac(int32_t acc, int32_t a, int32_t b) {
    return __viaddmax_s32(a, b, acc);
  }
  static __device__ __forceinline__ int32_t mac2(int32_t acc, int32_t a0, int32_t a1, int32_t b0, int32_t b1) {
    return __viaddmax_s32(a1, b1, __viaddmax_s32(a0, b0, acc));
  }
  static __device__ __forceinline__ int32_t mx(int32_t a, int32_t b) { return max(a, b); }
  static __device__ __forceinline__ int32_t from_w(float w) { return (int32_t)w; }
  // values at or below half the sentinel stand for -inf
  static __device__ __forceinline__ float to_f(int32_t v) {
    return v <= -268435456 ? __int_as_float(0xff800000) : (float)v;
  }
};

template <typename T>
struct Vec4;
template <>
struct Vec4<float> { using type = float4; };
template <>
struct Vec4<int32_t> { using type = int4; };
template <typename T>
struct Vec2;
template <>
struct Vec2<float> { using type = float2; };
template <>
struct Vec2<int32_t> { using type = int2; };

// Wait for the grid this one depends on programmatically (the previous
// per-level launch) to complete and its memory to be visible; returns at
// once after the first call, and in launches without that dependency.
// Every read or write of the arena in a per-level launch comes after it.
__device__ __forceinline__ void dep_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ int ld_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// ---------------------------------------------------------------------------
// leaves
// ---------------------------------------------------------------------------
template <typename T>
__device__ void leaves_tile(const LeafDesc* __restrict__ leaves, int n_leaves,
                            const int8_t* __restrict__ slice_vals, T* __restrict__ arena, int tile,
                            const float* __restrict__ weights) {
  int i = tile * kThreads + threadIdx.x;
  if (i >= n_leaves) return;
  const LeafDesc ld = leaves[i];
  const int nout = 1 << ld.n_out;
  const T w = Trop<T>::from_w(weights && ld.label >= 0 ? weights[ld.label] : ld.w);
  for (int e = 0; e < nout; e++) {
    T best = Trop<T>::neg();
    for (int raw = 0; raw < (1 << ld.nraw); raw++) {
      bool ok = true;
      for (int k = 0; k < ld.nraw; k++) {
        int x = (raw >> k) & 1;
        if (ld.slice_idx[k] >= 0) {
          if (x != (int)slice_vals[ld.slice_idx[k]]) ok = false;
        } else if (((e >> ld.out_bit[k]) & 1) != x) {
          ok = false;
        }
      }
      if (!ok) continue;
      T v;
      if (ld.nraw == 1) v = (raw & 1) ? w : T(0);
      else v = (raw == 3) ? Trop<T>::neg() : T(0);
      best = Trop<T>::mx(best, v);
    }
    arena[ld.off + e] = best;
  }
}

// ---------------------------------------------------------------------------
// stream tile
// ---------------------------------------------------------------------------
// XOR swizzle of a shared-memory word index at 16-byte granularity: bits 2..4
// of the index are XORed with bits 5..7 and 10..12.  It is linear over GF(2)
// (the swizzle of an OR of disjoint bit fields is the XOR of their swizzles),
// keeps every aligned 4-word chunk contiguous (so 16-byte async copies land
// intact) and spreads power-of-two strides over 8 bank groups.
__host__ __device__ __forceinline__ int swz16(int j) { return j ^ ((((j >> 5) ^ (j >> 10)) & 7) << 2); }

// Operand regions are padded to 4 words so every 16-byte async copy lands on
// a 16-byte boundary of shared memory.
__host__ __device__ inline int stream_a_words(const TileDesc& d) { return ((1 << d.na) + 3) & ~3; }
__host__ __device__ inline int stream_buf_words(const TileDesc& d) {
  return stream_a_words(d) + (d.b_off >= 0 ? (((1 << d.nb) + 3) & ~3) : 0);
}
// Pipeline depth: as many operand buffers as fit in the staging area of two
// full-size buffers, from 2 (operand tiles of 2^13 words) up to kMaxStages
// (short tiles, where the bytes in flight would otherwise be too few to cover
// the memory latency).
__host__ __device__ inline int stream_stages(const TileDesc& d) {
  const int s = (2 * kSmemFloats) / stream_buf_words(d);
  return s < 2 ? 2 : s > kMaxStages ? kMaxStages : s;
}
// shared memory of a stream tile: the descriptor, the operand buffers, then
// tables
__host__ __device__ inline int stream_smem_words(const TileDesc& d) {
  const bool hasB = d.b_off >= 0;
  int w = kDescWords + stream_stages(d) * stream_buf_words(d);
  w += 1 << (d.na - d.pa);
  w += hasB ? (1 << (d.nb - d.pb)) : 0;
  w += 1 << (d.n_tc - d.pc);
  w += 2 * (1 << d.n_tr);
  w += kThreads;
  w += 5 * kMaxBits;  // offset increments
  return w;
}
// upper bound of stream_smem_words over every descriptor plan_tile emits
__host__ __device__ constexpr int stream_smem_words_max() {
  return kDescWords + 2 * kSmemFloats + 3 * 512 + 2 * 256 + kThreads + 5 * kMaxBits;
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async8(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst)), "l"(src)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// wait until at most n (0..7) committed groups are pending
__device__ __forceinline__ void cp_async_wait_n(int n) {
  switch (n) {
    case 7: cp_async_wait<7>(); break;
    case 6: cp_async_wait<6>(); break;
    case 5: cp_async_wait<5>(); break;
    case 4: cp_async_wait<4>(); break;
    case 3: cp_async_wait<3>(); break;
    case 2: cp_async_wait<2>(); break;
    case 1: cp_async_wait<1>(); break;
    default: cp_async_wait<0>(); break;
  }
}

// Issue async copies of the 2^n-element sub-tensor at src into swizzled
// shared memory (tile bit b <-> tensor position pos[b]; bits below p are the
// tensor's positions 0..p-1, the rest go through the table hi).
template <typename T>
__device__ __forceinline__ void issue_sub(T* __restrict__ dst, const T* __restrict__ src, int n, int p,
                                          const int* __restrict__ hi) {
  const int N = 1 << n;
  if (p >= 2) {
    const int lowmask = (1 << p) - 1;
    for (int q = threadIdx.x; q < (N >> 2); q += kThreads) {
      const int j = q << 2;
      cp_async16(dst + swz16(j), src + ((j & lowmask) + hi[j >> p]));
    }
  } else if (p == 1) {
    for (int q = threadIdx.x; q < (N >> 1); q += kThreads) {
      const int j = q << 1;
      cp_async8(dst + swz16(j), src + hi[j >> 1]);
    }
  } else {
    for (int j = threadIdx.x; j < N; j += kThreads) cp_async4(dst + swz16(j), src + hi[j]);
  }
}

// Per-CTA state of a run of stream tiles: shared-memory tables, the
// thread's fixed indices and the copy / compute / store cursors.
constexpr int kPreChunks = 2;  // 16-byte copies per thread and operand with precomputed offsets

template <typename T, bool PRE>
struct StreamRun {
  T* buf0;
  const int* ldA;
  const int* ldB;
  const int* stC;
  const int* IAr;
  const int* IBr;
  T* red;
  const int* incAg;
  const int* incBg;
  const int* incCg;
  const int* incAl;
  const int* incBl;
  const T* A0;
  const T* B0;
  T* C0;
  int NA, BUF, S;
  int na, pa, nb, pb, pc;
  int nloop, ntr, lo_bits, split, opt;
  bool hasB, act;
  int cl, s;
  int iah[kMaxOpt], ibh[kMaxOpt];
  int64_t n_items;
  // prefetch cursor (tile pt, loop step pr) and its operand offsets
  int64_t issued;
  uint32_t pt;  // tile indices fit 32 bits (TileDesc::n_tiles is an int32)
  int pr, pa_g, pb_g, pa_l, pb_l, ib;
  // compute / store cursor
  uint32_t ct;
  int oc, cb, rl;
  // 16-byte copies whose per-thread source and destination offsets are fixed
  // for the run (all but the item's base): computed once, when both operands
  // go by 16-byte chunks and each thread has at most kPreChunks of each.
  // Only the 128-register forms (PRE) keep the offsets: at 80 registers
  // they spill and cost more than they save.
  bool pre;
  int nca, ncb;
  int a_src[kPreChunks], a_dst[kPreChunks], b_src[kPreChunks], b_dst[kPreChunks];

  __device__ __forceinline__ void issue() {
    T* dst = buf0 + ib * BUF;
    if (PRE && pre) {
      const T* sa = A0 + (pa_g + pa_l);
#pragma unroll
      for (int k = 0; k < kPreChunks; k++)
        if (k < nca) cp_async16(dst + a_dst[k], sa + a_src[k]);
      if (hasB) {
        const T* sb = B0 + (pb_g + pb_l);
        T* db = dst + NA;
#pragma unroll
        for (int k = 0; k < kPreChunks; k++)
          if (k < ncb) cp_async16(db + b_dst[k], sb + b_src[k]);
      }
    } else {
      issue_sub<T>(dst, A0 + (pa_g + pa_l), na, pa, ldA);
      if (hasB) issue_sub<T>(dst + NA, B0 + (pb_g + pb_l), nb, pb, ldB);
    }
    ib = ib + 1 == S ? 0 : ib + 1;
    if (pr + 1 < nloop) {
      const int k = __ffs(~pr) - 1;
      pa_l += incAl[k];
      pb_l += incBl[k];
      pr++;
    } else {
      pr = 0;
      pa_l = pb_l = 0;
      const int k = __ffs(~pt) - 1;
      pa_g += incAg[k];
      pb_g += incBg[k];
      pt++;
    }
    issued++;
  }
  // item `issued` into the buffer freed by the item before the current one
  __device__ __forceinline__ void refill() {
    if (issued < n_items) issue();
    cp_async_commit();
  }
  template <int N = kMaxOpt>
  __device__ __forceinline__ void store(const T* acc) {
    const int cmask = (1 << pc) - 1;
    T* Ct = C0 + oc;
#pragma unroll
    for (int i = 0; i < N; i++) {
      if (i < opt) {
        if constexpr (PRE) {
          Ct[st_off[i]] = acc[i];
        } else {
          const int c = cl + (i << lo_bits);
          Ct[(c & cmask) + stC[c >> pc]] = acc[i];
        }
      }
    }
  }
  // the thread's output offsets within a tile (fixed for the run)
  int st_off[PRE ? kMaxOpt : 1];
  __device__ __forceinline__ void next_tile() {
    const int k = __ffs(~ct) - 1;
    oc += incCg[k];
    ct++;
  }
};

// The loop for the common shape: two operands, no reduction split, OPT
// outputs per thread and NTR in-tile reduction terms, all compile-time.
// One barrier per item: after it, item `it` is visible to every thread and
// every thread is done with item it - 1, whose buffer the refill reuses.
// In-tile reduction offsets are XORs of one basis offset per reduced bit
// (the swizzle is linear over GF(2)): the terms are visited in Gray-code
// order, one XOR per step, so only log2(NTR) offsets per operand stay in
// registers.
// Terms are packed in pairs (pack2 + add.f32x2 + 3-input max) from this many
// in-tile reduction terms on; fewer go one add and one max each.
constexpr int kPairMin = 8;

template <typename T, int OPT, int NTR, bool PRE>
__device__ __forceinline__ void stream_loop_fixed(StreamRun<T, PRE>& R) {
  constexpr int LTR = NTR >= 16 ? 4 : NTR >= 8 ? 3 : NTR >= 4 ? 2 : NTR >= 2 ? 1 : 0;
  static_assert((1 << LTR) == NTR, "NTR is a power of two");
  int ba[LTR > 0 ? LTR : 1], bb[LTR > 0 ? LTR : 1];
#pragma unroll
  for (int b = 0; b < LTR; b++) {
    ba[b] = R.IAr[1 << b];
    bb[b] = R.IBr[1 << b];
  }
  T acc[OPT];
#pragma unroll
  for (int i = 0; i < OPT; i++) acc[i] = Trop<T>::neg();
  const int last = R.nloop - 1;
  for (int64_t it = 0; it < R.n_items; it++) {
    cp_async_wait_n(R.S - 2);
    __syncthreads();
    R.refill();
    const T* As = R.buf0 + R.cb * R.BUF;
    const T* Bs = As + R.NA;
    R.cb = R.cb + 1 == R.S ? 0 : R.cb + 1;
    if (R.act) {
#pragma unroll
      for (int i = 0; i < OPT; i++) {
        int xa = R.iah[i], xb = R.ibh[i];  // term 0: the reduced bits' offsets are 0
        if constexpr (NTR == 1) {
          acc[i] = Trop<T>::mac(acc[i], As[xa], Bs[xb]);
        } else {
          // two independent chains for NTR >= 4
          T a0 = acc[i], a1 = Trop<T>::neg();
#pragma unroll
          for (int r = 0; r < NTR; r += 2) {
            // the pair (g, g ^ bit 0) of Gray-code terms
            const T x0 = As[xa], y0 = Bs[xb];
            const T x1 = As[xa ^ ba[0]], y1 = Bs[xb ^ bb[0]];
            T& a = (NTR >= 4 && (r & 2)) ? a1 : a0;
            if constexpr (NTR >= kPairMin) a = Trop<T>::mac2(a, x0, x1, y0, y1);
            else a = Trop<T>::mac(Trop<T>::mac(a, x0, y0), x1, y1);
            if (r + 2 < NTR) {
              // pair index m = r / 2 moves to m + 1: flip reduced bit
              // 1 + ctz(m + 1) = ctz(r + 2)
              const int k = __ffs(r + 2) - 1;
              xa ^= ba[k];
              xb ^= bb[k];
            }
          }
          acc[i] = NTR >= 4 ? Trop<T>::mx(a0, a1) : a0;
        }
      }
    }
    if (R.rl == last) {
      if (R.act) R.template store<OPT>(acc);
#pragma unroll
      for (int i = 0; i < OPT; i++) acc[i] = Trop<T>::neg();
      R.next_tile();
      R.rl = 0;
    } else {
      R.rl++;
    }
  }
}

// Any shape: unary nodes, reduction splits, longer in-tile reductions.
// MAXOPT bounds the outputs per thread (1 for tiles of <= 256 outputs).
template <typename T, int MAXOPT, bool PRE>
__device__ __forceinline__ void stream_loop_any(StreamRun<T, PRE>& R) {
  const int t = threadIdx.x;
  T acc[MAXOPT];
#pragma unroll
  for (int i = 0; i < MAXOPT; i++) acc[i] = Trop<T>::neg();
  const int step = 1 << R.split;
  const int last = R.nloop - 1;
  for (int64_t it = 0; it < R.n_items; it++) {
    cp_async_wait_n(R.S - 2);
    __syncthreads();
    R.refill();
    const T* As = R.buf0 + R.cb * R.BUF;
    const T* Bs = As + R.NA;
    R.cb = R.cb + 1 == R.S ? 0 : R.cb + 1;
    if (R.act) {
#pragma unroll
      for (int i = 0; i < MAXOPT; i++) {
        if (i < R.opt) {
          T a = acc[i];
          const int ia = R.iah[i], ib = R.ibh[i];
          if (R.hasB) {
            for (int r = R.s; r < R.ntr; r += step) a = Trop<T>::mac(a, As[ia ^ R.IAr[r]], Bs[ib ^ R.IBr[r]]);
          } else {
            for (int r = R.s; r < R.ntr; r += step) a = Trop<T>::mx(a, As[ia ^ R.IAr[r]]);
          }
          acc[i] = a;
        }
      }
    }
    if (R.rl == last) {
      if (R.split > 0) {
        // red[] of the previous tile was read before this item's barrier
        R.red[t] = acc[0];
        __syncthreads();
        if (R.act && R.s == 0) {
          T a = acc[0];
          for (int s2 = 1; s2 < step; s2++) a = Trop<T>::mx(a, R.red[R.cl + (s2 << R.lo_bits)]);
          acc[0] = a;
        }
      }
      if (R.act && R.s == 0) R.template store<MAXOPT>(acc);
#pragma unroll
      for (int i = 0; i < MAXOPT; i++) acc[i] = Trop<T>::neg();
      R.next_tile();
      R.rl = 0;
    } else {
      R.rl++;
    }
  }
}

// Run tiles [t0, t1) of one stream-tile descriptor on this CTA: the
// descriptor is copied to shared memory and the index tables built from it
// once, and the operand sub-tiles of the next stream_stages(d) - 1 (tile,
// loop step) items are copied asynchronously while the current one is
// reduced.
template <typename T, bool PRE = false>
__device__ void stream_tiles(const TileDesc& dg, int64_t t0, int64_t t1, T* __restrict__ arena,
                             int* __restrict__ smem, int* err = nullptr) {
  (void)err;  // the per-thread copy pipeline has no waits to bound
  const int t = threadIdx.x;
  __syncthreads();  // the previous user of this shared memory is done
  {
    const int* src = reinterpret_cast<const int*>(&dg);
    for (int j = t; j < (int)(sizeof(TileDesc) / 4); j += kThreads) smem[j] = src[j];
  }
  __syncthreads();
  const TileDesc& d = *reinterpret_cast<const TileDesc*>(smem);
  StreamRun<T, PRE> R;
  R.hasB = d.b_off >= 0;
  R.NA = stream_a_words(d);  // A region (padded), B region follows
  R.BUF = stream_buf_words(d);
  R.S = stream_stages(d);
  R.na = d.na;
  R.pa = d.pa;
  R.nb = d.nb;
  R.pb = d.pb;
  R.pc = d.pc;
  T* buf0 = reinterpret_cast<T*>(smem + kDescWords);
  R.buf0 = buf0;
  int* ldA = reinterpret_cast<int*>(buf0 + R.S * R.BUF);
  const int nAh = 1 << (d.na - d.pa);
  const int nBh = R.hasB ? (1 << (d.nb - d.pb)) : 0;
  const int nCh = 1 << (d.n_tc - d.pc);
  const int ntr = 1 << d.n_tr;
  int* ldB = ldA + nAh;
  int* stC = ldB + nBh;
  int* IAr = stC + nCh;
  int* IBr = IAr + ntr;
  T* red = reinterpret_cast<T*>(IBr + ntr);
  // increments of the grid / loop offsets when the index goes from x to x+1
  // with k trailing ones: +2^pos_k - sum_{i<k} 2^pos_i (pos -1: no term)
  int* incAg = reinterpret_cast<int*>(red + kThreads);
  for (int j = t; j < nAh; j += kThreads) {
    int o = 0;
    for (int b = 0; b < d.na - d.pa; b++)
      if ((j >> b) & 1) o += 1 << d.ta_pos[d.pa + b];
    ldA[j] = o;
  }
  for (int j = t; j < nBh; j += kThreads) {
    int o = 0;
    for (int b = 0; b < d.nb - d.pb; b++)
      if ((j >> b) & 1) o += 1 << d.tb_pos[d.pb + b];
    ldB[j] = o;
  }
  for (int j = t; j < nCh; j += kThreads) {
    int o = 0;
    for (int b = 0; b < d.n_tc - d.pc; b++)
      if ((j >> b) & 1) o += 1 << d.tc_pos[d.pc + b];
    stC[j] = o;
  }
  for (int j = t; j < ntr; j += kThreads) {
    int xa = 0, xb = 0;
    for (int b = 0; b < d.n_tr; b++) {
      if ((j >> b) & 1) {
        if (d.tr_a[b] >= 0) xa |= 1 << d.tr_a[b];
        if (d.tr_b[b] >= 0) xb |= 1 << d.tr_b[b];
      }
    }
    IAr[j] = swz16(xa);
    IBr[j] = swz16(xb);
  }
  if (t < 5 * kMaxBits) {
    const int which = t / kMaxBits, k = t % kMaxBits;
    const int nbits = which < 3 ? d.n_grid : d.n_loop;
    const int8_t* pos = which == 0 ? d.g_pa : which == 1 ? d.g_pb : which == 2 ? d.g_pc : which == 3 ? d.l_pa : d.l_pb;
    int v = 0;
    if (k < nbits) {
      if (pos[k] >= 0) v += 1 << pos[k];
      for (int i = 0; i < k; i++)
        if (pos[i] >= 0) v -= 1 << pos[i];
    }
    incAg[which * kMaxBits + k] = v;
  }
  R.ldA = ldA;
  R.ldB = ldB;
  R.stC = stC;
  R.IAr = IAr;
  R.IBr = IBr;
  R.red = red;
  R.incAg = incAg;
  R.incBg = incAg + kMaxBits;
  R.incCg = incAg + 2 * kMaxBits;
  R.incAl = incAg + 3 * kMaxBits;
  R.incBl = incAg + 4 * kMaxBits;

  // thread -> (output, reduction split)
  R.lo_bits = d.n_tc < 8 ? d.n_tc : 8;
  R.split = d.split_log2;
  const int active = 1 << (R.lo_bits + R.split);
  R.opt = 1 << (d.n_tc - R.lo_bits);
  R.act = t < active;
  R.cl = t & ((1 << R.lo_bits) - 1);
  R.s = t >> R.lo_bits;
  R.ntr = ntr;
  int iat = 0, ibt = 0;
  for (int b = 0; b < R.lo_bits; b++) {
    if ((R.cl >> b) & 1) {
      if (d.tc_a[b] >= 0) iat |= 1 << d.tc_a[b];
      if (d.tc_b[b] >= 0) ibt |= 1 << d.tc_b[b];
    }
  }
  iat = swz16(iat);
  ibt = swz16(ibt);
#pragma unroll
  for (int i = 0; i < kMaxOpt; i++) {
    int xa = 0, xb = 0;
    if (i < R.opt) {
      for (int b = R.lo_bits; b < d.n_tc; b++) {
        if (((i << R.lo_bits) >> b) & 1) {
          if (d.tc_a[b] >= 0) xa |= 1 << d.tc_a[b];
          if (d.tc_b[b] >= 0) xb |= 1 << d.tc_b[b];
        }
      }
    }
    R.iah[i] = iat ^ swz16(xa);
    R.ibh[i] = ibt ^ swz16(xb);
  }
  // absolute grid offsets of the first tile (32-bit within each tensor)
  int ga = 0, gb = 0, gc = 0;
  for (int i = 0; i < d.n_grid; i++) {
    if ((t0 >> i) & 1) {
      if (d.g_pa[i] >= 0) ga += 1 << d.g_pa[i];
      if (d.g_pb[i] >= 0) gb += 1 << d.g_pb[i];
      gc += 1 << d.g_pc[i];
    }
  }
  R.nloop = 1 << d.n_loop;
  R.n_items = (t1 - t0) * R.nloop;
  R.A0 = arena + d.a_off;
  R.B0 = arena + (R.hasB ? d.b_off : 0);
  R.C0 = arena + d.c_off;
  R.pt = (uint32_t)t0;
  R.issued = 0;
  R.pr = 0;
  R.pa_g = ga;
  R.pb_g = gb;
  R.pa_l = R.pb_l = 0;
  R.ib = 0;
  R.ct = (uint32_t)t0;
  R.oc = gc;
  R.cb = 0;
  R.rl = 0;
  const bool fixed = R.hasB && R.split == 0 && ntr <= 16;
  const int shape = R.opt * 32 + ntr;
  __syncthreads();  // tables ready
  if constexpr (PRE) {
    const int cmask = (1 << d.pc) - 1;
#pragma unroll
    for (int i = 0; i < kMaxOpt; i++) {
      const int c = R.cl + (i << R.lo_bits);
      R.st_off[i] = i < R.opt ? (c & cmask) + stC[c >> d.pc] : 0;
    }
  }
  {
    const int ca = (1 << d.na) >> 2, cbn = R.hasB ? (1 << d.nb) >> 2 : 0;
    R.pre = PRE && d.pa >= 2 && ca <= kPreChunks * kThreads &&
            (!R.hasB || (d.pb >= 2 && cbn <= kPreChunks * kThreads));
    R.nca = R.ncb = 0;
#pragma unroll
    for (int k = 0; k < kPreChunks; k++) {
      R.a_src[k] = R.a_dst[k] = R.b_src[k] = R.b_dst[k] = 0;
      const int q = t + k * kThreads, j = q << 2;
      if (R.pre && q < ca) {
        R.a_dst[k] = swz16(j);
        R.a_src[k] = (j & ((1 << d.pa) - 1)) + ldA[j >> d.pa];
        R.nca = k + 1;
      }
      if (R.pre && q < cbn) {
        R.b_dst[k] = swz16(j);
        R.b_src[k] = (j & ((1 << d.pb) - 1)) + ldB[j >> d.pb];
        R.ncb = k + 1;
      }
    }
  }
  // prologue: items 0 .. S-2, one commit group each (empty past the end);
  // the arena's first access (the tables above read only the descriptor)
  dep_wait();
  for (int k = 0; k < R.S - 1; k++) R.refill();
  if (fixed) {
    switch (shape) {
      case 1 * 32 + 1: stream_loop_fixed<T, 1, 1, PRE>(R); break;
      case 1 * 32 + 2: stream_loop_fixed<T, 1, 2, PRE>(R); break;
      case 1 * 32 + 4: stream_loop_fixed<T, 1, 4, PRE>(R); break;
      case 1 * 32 + 8: stream_loop_fixed<T, 1, 8, PRE>(R); break;
      case 1 * 32 + 16: stream_loop_fixed<T, 1, 16, PRE>(R); break;
      case 2 * 32 + 1: stream_loop_fixed<T, 2, 1, PRE>(R); break;
      case 2 * 32 + 2: stream_loop_fixed<T, 2, 2, PRE>(R); break;
      case 2 * 32 + 4: stream_loop_fixed<T, 2, 4, PRE>(R); break;
      case 2 * 32 + 8: stream_loop_fixed<T, 2, 8, PRE>(R); break;
      case 2 * 32 + 16: stream_loop_fixed<T, 2, 16, PRE>(R); break;
      case 4 * 32 + 1: stream_loop_fixed<T, 4, 1, PRE>(R); break;
      case 4 * 32 + 2: stream_loop_fixed<T, 4, 2, PRE>(R); break;
      case 4 * 32 + 4: stream_loop_fixed<T, 4, 4, PRE>(R); break;
      case 4 * 32 + 8: stream_loop_fixed<T, 4, 8, PRE>(R); break;
      case 4 * 32 + 16: stream_loop_fixed<T, 4, 16, PRE>(R); break;
      case 8 * 32 + 1: stream_loop_fixed<T, 8, 1, PRE>(R); break;
      case 8 * 32 + 2: stream_loop_fixed<T, 8, 2, PRE>(R); break;
      case 8 * 32 + 4: stream_loop_fixed<T, 8, 4, PRE>(R); break;
      case 8 * 32 + 8: stream_loop_fixed<T, 8, 8, PRE>(R); break;
      default:
        if (R.opt == 1) stream_loop_any<T, 1, PRE>(R);
        else stream_loop_any<T, kMaxOpt, PRE>(R);
        break;
    }
  } else if (R.opt == 1) {
    stream_loop_any<T, 1, PRE>(R);
  } else {
    stream_loop_any<T, kMaxOpt, PRE>(R);
  }
  cp_async_wait<0>();
}

// A tiny stream step (Group::tiny) by one warp, straight from global memory
// (its operands are a few hundred bytes, so staging would cost more than the
// reads).  Lane l takes reduced term r = l mod 2^n_tr of output l >> n_tr of
// each pass (32 >> n_tr outputs a pass); the loads of four passes are in
// flight at once, then the terms of each output meet in a shuffle max and
// lane r = 0 stores it.  An offset is the sum of one power of two per set
// bit of the output and term indices (distinct tensor positions).
constexpr int kTinyPassesAtOnce = 4;

template <typename T>
__device__ __noinline__ void tiny_node(const TinyDesc* __restrict__ dp, T* __restrict__ arena) {
  const int lane = threadIdx.x & 31;
  const TinyDesc d = *dp;
  const int n_tc = d.n_tc, n_tr = d.n_tr;
  const bool hasB = d.b_off >= 0;
  const T* A = arena + d.a_off;
  const T* B = arena + (hasB ? d.b_off : 0);
  T* C = arena + d.c_off;
  const int r = lane & ((1 << n_tr) - 1);
  int ra = 0, rb = 0;
#pragma unroll
  for (int b = 0; b < kTinyRed; b++)
    if (b < n_tr && ((r >> b) & 1)) {
      if (d.ra[b] >= 0) ra += 1 << d.ra[b];
      if (d.rb[b] >= 0) rb += 1 << d.rb[b];
    }
  const int n_out = 1 << n_tc, per = 32 >> n_tr;
  const int passes = (n_out + per - 1) / per;
  for (int p0 = 0; p0 < passes; p0 += kTinyPassesAtOnce) {  // the same trip count on every lane
    T v[kTinyPassesAtOnce];
    int oc[kTinyPassesAtOnce];
#pragma unroll
    for (int k = 0; k < kTinyPassesAtOnce; k++) {
      const int c = (p0 + k) * per + (lane >> n_tr);
      v[k] = Trop<T>::neg();
      oc[k] = 0;
      if (p0 + k < passes && c < n_out) {
        int oa = ra, ob = rb;
#pragma unroll
        for (int b = 0; b < kTinyOut; b++)
          if (b < n_tc && ((c >> b) & 1)) {
            if (d.oa[b] >= 0) oa += 1 << d.oa[b];
            if (d.ob[b] >= 0) ob += 1 << d.ob[b];
            oc[k] += 1 << d.oc[b];
          }
        v[k] = hasB ? Trop<T>::mac(v[k], __ldcg(A + oa), __ldcg(B + ob)) : __ldcg(A + oa);
      }
    }
#pragma unroll
    for (int k = 0; k < kTinyPassesAtOnce; k++) {
      if (p0 + k < passes) {  // warp-uniform
        T x = v[k];
        for (int s = 1; s < (1 << n_tr); s <<= 1) x = Trop<T>::mx(x, __shfl_xor_sync(0xffffffffu, x, s));
        const int c = (p0 + k) * per + (lane >> n_tr);
        if (r == 0 && c < n_out) C[oc[k]] = x;
      }
    }
  }
}

// One tile (the launch-per-tile form used by the plain path's kernels).
template <typename T>
__device__ __forceinline__ void stream_tile(const TileDesc& d, int64_t tile, T* __restrict__ arena,
                                            int* __restrict__ smem) {
  stream_tiles<T>(d, tile, tile + 1, arena, smem);
}

// ---------------------------------------------------------------------------
// final: max over the root tensor, + r
// ---------------------------------------------------------------------------
template <typename T>
__device__ void final_tile(const FinalDesc& f, const T* __restrict__ arena, float r, float* out) {
  __shared__ float wmax[kThreads / 32];
  const int64_t n = int64_t(1) << f.root_log2;
  T m = Trop<T>::neg();
  for (int64_t i = threadIdx.x; i < n; i += kThreads) m = Trop<T>::mx(m, __ldcg(arena + f.root_off + i));
  float v = Trop<T>::to_f(m);
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    float b = wmax[0];
    for (int w = 1; w < kThreads / 32; w++) b = fmaxf(b, wmax[w]);
    *out = b + r;
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// K1: batched max-plus GEMM, canonical column-major operands
//   C[m + M n + MN b] = max_k A[m + M k + MK b] + B[k + K n + KN b]
// CTA tile BM x BN, BK = 16 per stage, 256 threads in a 16 x 16 grid, each
// owning a TM x TN register tile (TM = BM / 16, TN = BN / 16).  Shared memory
// keeps k in interleaved pairs, so one 64-bit load yields (x[k], x[k+1]) and
// the inner step is one add.f32x2 and one three-input max.f32 per two MACs.
// ---------------------------------------------------------------------------

template <typename T, int BM, int BN>
struct K1Cfg {
  static constexpr int BK = 16;
  static constexpr int TM = BM / 16, TN = BN / 16;
  static constexpr int A_WORDS = BK * BM, B_WORDS = BK * BN;
  static constexpr int SMEM_BYTES = 2 * (A_WORDS + B_WORDS) * (int)sizeof(T);
};

// Thread layout of the 256-thread GEMM tiles: 8 warps as 2 (m) x 4 (n), each
// warp 8 (m) x 4 (n) lanes, each thread a TM x TN register tile split in two
// halves per dimension.  A warp reads 8 m-groups and 4 n-groups per k pair,
// which keeps shared-memory traffic near 96 B/clk/SM at full issue rate.
// Rows of a thread: two halves of H rows; within a half, pairs of rows sit at
// lm * 2 so the 8 m-lanes of a warp read 8 consecutive 16-byte chunks (one
// conflict-free wavefront per 128-bit shared load).
// The skinny tiles (256 x 16, 16 x 256) instead give each thread a 4 x 4
// block of consecutive rows and columns: 64 groups along the long side (warp
// w, lanes >> 2) by 4 along the short one (lanes & 3), so every shared pair
// a thread loads serves four accumulators.
template <int BM, int BN>
struct GemmShape {
  static constexpr bool SKINNY_M = BM == 256 && BN == 16, SKINNY_N = BM == 16 && BN == 256;
  static constexpr int TM = SKINNY_M || SKINNY_N ? 4 : BM / 16;
  static constexpr int TN = SKINNY_M || SKINNY_N ? 4 : BN / 16;
  // (wm, wn, lm, ln) of gm_row / gm_col for thread lane of warp
  __host__ __device__ static constexpr int wm(int warp) { return SKINNY_M ? warp : SKINNY_N ? 0 : warp & 1; }
  __host__ __device__ static constexpr int wn(int warp) { return SKINNY_M ? 0 : SKINNY_N ? warp : warp >> 1; }
  __host__ __device__ static constexpr int lm(int lane) { return SKINNY_M ? lane >> 2 : SKINNY_N ? lane & 3 : lane & 7; }
  __host__ __device__ static constexpr int ln(int lane) { return SKINNY_M ? lane & 3 : SKINNY_N ? lane >> 2 : lane >> 3; }
};
template <int TM, int BM>
__host__ __device__ constexpr int gm_row(int wm, int lm, int i) {
  constexpr int H = TM >= 2 ? TM / 2 : 1;
  if constexpr (BM == 256 && TM == 4) {
    return (wm * 8 + lm) * 4 + i;  // skinny 256 x 16
  } else if constexpr (BM == 16 && TM == 4) {
    return lm * 4 + i;  // skinny 16 x 256
  } else if constexpr (H >= 2) {
    const int q = i % H;
    return wm * (BM / 2) + (i / H) * (BM / 4) + (q / 2) * 16 + lm * 2 + (q % 2);
  } else {
    return wm * (BM / 2) + (i / H) * (BM / 4) + lm;
  }
}
template <int TN, int BN>
__host__ __device__ constexpr int gm_col(int wn, int ln, int j) {
  constexpr int H = TN >= 2 ? TN / 2 : 1;
  if constexpr (BN == 16 && TN == 4) {
    return ln * 4 + j;  // skinny 256 x 16
  } else if constexpr (BN == 256 && TN == 4) {
    return (wn * 8 + ln) * 4 + j;  // skinny 16 x 256
  } else {
    return wn * (BN / 4) + (j / H) * (BN / 8) + ln * H + (j % H);
  }
}
// Every (row, column) of a BM x BN tile is one thread's accumulator exactly
// once, and a thread's rows i, i + 1 (i even) are adjacent when TM >= 4 (the
// paired stores of the epilogue rely on it).
template <int BM, int BN>
__host__ __device__ constexpr bool gm_covers() {
  using G = GemmShape<BM, BN>;
  constexpr int TM = G::TM, TN = G::TN;
  if (TM * TN * 256 != BM * BN) return false;
  bool seen[BM * BN] = {};
  for (int t = 0; t < 256; t++)
    for (int i = 0; i < TM; i++)
      for (int j = 0; j < TN; j++) {
        const int r = gm_row<TM, BM>(G::wm(t >> 5), G::lm(t & 31), i);
        const int c = gm_col<TN, BN>(G::wn(t >> 5), G::ln(t & 31), j);
        if (r < 0 || r >= BM || c < 0 || c >= BN || seen[r * BN + c]) return false;
        seen[r * BN + c] = true;
        if (TM >= 4 && i % 2 == 0 && gm_row<TM, BM>(G::wm(t >> 5), G::lm(t & 31), i + 1) != r + 1) return false;
      }
  return true;
}

// One k-pair step of the register tile: shared tiles hold [kp][x][2].  The
// a-pairs are loaded per half so that at most 64 accumulators + 4 a-pairs +
// TN b-pairs are live.
template <typename T, int TM, int TN, int BM, int BN>
__device__ __forceinline__ void mp_step(const T* __restrict__ as, const T* __restrict__ bs, int kp, int wm,
                                        int wn, int lm, int ln, T (&acc)[TM][TN]) {
  uint64_t b2[TN];
#pragma unroll
  for (int j = 0; j < TN; j++)
    b2[j] = *reinterpret_cast<const uint64_t*>(bs + (kp * BN + gm_col<TN, BN>(wn, ln, j)) * 2);
  constexpr int HM = TM >= 2 ? TM / 2 : 1;
#pragma unroll
  for (int h = 0; h < TM; h += HM) {
    uint64_t a2[HM];
#pragma unroll
    for (int i = 0; i < HM; i++)
      a2[i] = *reinterpret_cast<const uint64_t*>(as + (kp * BM + gm_row<TM, BM>(wm, lm, h + i)) * 2);
    if constexpr (std::is_same<T, float>::value) {
#pragma unroll
      for (int i = 0; i < HM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) {
          uint64_t s2 = add2(a2[i], b2[j]);
          acc[h + i][j] = max3(acc[h + i][j], lo32(s2), hi32(s2));
        }
    } else {
#pragma unroll
      for (int i = 0; i < HM; i++)
#pragma unroll
        for (int j = 0; j < TN; j++) {
          int32_t x0 = (int32_t)(uint32_t)a2[i], x1 = (int32_t)(uint32_t)(a2[i] >> 32);
          int32_t y0 = (int32_t)(uint32_t)b2[j], y1 = (int32_t)(uint32_t)(b2[j] >> 32);
          T v = Trop<T>::mac(acc[h + i][j], (T)x0, (T)y0);
          acc[h + i][j] = Trop<T>::mac(v, (T)x1, (T)y1);
        }
    }
  }
}

// Packed-int16 form of one k-pair step: shared tiles hold [kp][x] words of
// (x[k], x[k+1]) as two int16; __viaddmax_s16x2 adds the pairs and keeps the
// even-k and odd-k maxima in the two halves of the accumulator.
template <int TM, int TN, int BM, int BN>
__device__ __forceinline__ void mp_step_i16(const uint32_t* __restrict__ as, const uint32_t* __restrict__ bs, int kp,
                                            int wm, int wn, int lm, int ln, uint32_t (&acc)[TM][TN]) {
  uint32_t b[TN];
#pragma unroll
  for (int j = 0; j < TN; j++) b[j] = bs[kp * BN + gm_col<TN, BN>(wn, ln, j)];
#pragma unroll
  for (int i = 0; i < TM; i++) {
    const uint32_t a = as[kp * BM + gm_row<TM, BM>(wm, lm, i)];
#pragma unroll
    for (int j = 0; j < TN; j++) acc[i][j] = __viaddmax_s16x2(a, b[j], acc[i][j]);
  }
}

// Exact int16 stand-ins for the tropical values of an MIS network whose
// weights are integers >= 0 summing below 8192: every finite value is an
// integer in [0, 8191], -inf becomes -8192, a sum involving it stays negative
// and a sum of finite values stays below 16384.
constexpr int kI16Neg = -8192;
__device__ __forceinline__ uint32_t pack_i16(float x0, float x1) {
  const int v0 = __float2int_rz(fmaxf(x0, (float)kI16Neg));
  const int v1 = __float2int_rz(fmaxf(x1, (float)kI16Neg));
  return (uint32_t)(v0 & 0xffff) | ((uint32_t)v1 << 16);
}
__device__ __forceinline__ float unpack_max_i16(uint32_t acc) {
  const int lo = (int)(int16_t)(acc & 0xffffu), hi = (int)(int16_t)(acc >> 16);
  const int m = lo > hi ? lo : hi;
  return m < 0 ? __int_as_float(0xff800000) : (float)m;
}

template <typename T, int BM, int BN>
__global__ void __launch_bounds__(256) gemm_k1(const T* __restrict__ A, const T* __restrict__ B,
                                               T* __restrict__ C, int M, int N, int K, int64_t tiles_mn) {
  using Cfg = K1Cfg<T, BM, BN>;
  constexpr int BK = Cfg::BK, TM = Cfg::TM, TN = Cfg::TN;
  extern __shared__ __align__(16) unsigned char k1_smem[];
  T* As = reinterpret_cast<T*>(k1_smem);          // [2][BK/2][BM][2]
  T* Bs = As + 2 * Cfg::A_WORDS;                  // [2][BK/2][BN][2]
  const int t = threadIdx.x;
  const int64_t blk = blockIdx.x;
  const int64_t bat = blk / tiles_mn;
  const int64_t mn = blk % tiles_mn;
  const int tiles_m = M / BM;
  const int m0 = (int)(mn % tiles_m) * BM, n0 = (int)(mn / tiles_m) * BN;
  const T* Ab = A + bat * (int64_t)M * K;
  const T* Bb = B + bat * (int64_t)K * N;
  T* Cb = C + bat * (int64_t)M * N;
  const int warp = t >> 5, lane = t & 31;
  const int wm = warp & 1, wn = warp >> 1, lm = lane & 7, ln = lane >> 3;

  // global -> register staging
  constexpr int A_GROUPS = (BM / 4) * (BK / 2);  // (4 m) x (k pair) groups
  constexpr int B_GROUPS = (BK / 4) * BN;         // (4 k) x n groups
  constexpr int A_PER = (A_GROUPS + 255) / 256;
  constexpr int B_PER = (B_GROUPS + 255) / 256;
  using V4 = typename Vec4<T>::type;
  V4 ra0[A_PER], ra1[A_PER], rb[B_PER];
  auto gload = [&](int k0) {
#pragma unroll
    for (int u = 0; u < A_PER; u++) {
      int g = t + u * 256;
      if (g < A_GROUPS) {
        int m4 = g % (BM / 4), kp = g / (BM / 4);
        const T* p = Ab + (int64_t)(k0 + 2 * kp) * M + m0 + 4 * m4;
        ra0[u] = __ldg(reinterpret_cast<const V4*>(p));
        ra1[u] = __ldg(reinterpret_cast<const V4*>(p + M));
      }
    }
#pragma unroll
    for (int u = 0; u < B_PER; u++) {
      int g = t + u * 256;
      if (g < B_GROUPS) {
        int q = g % (BK / 4), n = g / (BK / 4);
        rb[u] = __ldg(reinterpret_cast<const V4*>(Bb + (int64_t)(n0 + n) * K + k0 + 4 * q));
      }
    }
  };
  auto sstore = [&](int buf) {
    T* as = As + buf * Cfg::A_WORDS;
    T* bs = Bs + buf * Cfg::B_WORDS;
#pragma unroll
    for (int u = 0; u < A_PER; u++) {
      int g = t + u * 256;
      if (g < A_GROUPS) {
        int m4 = g % (BM / 4), kp = g / (BM / 4);
        T* d = as + (kp * BM + 4 * m4) * 2;
        V4 x, y;
        x.x = ra0[u].x; x.y = ra1[u].x; x.z = ra0[u].y; x.w = ra1[u].y;
        y.x = ra0[u].z; y.y = ra1[u].z; y.z = ra0[u].w; y.w = ra1[u].w;
        reinterpret_cast<V4*>(d)[0] = x;
        reinterpret_cast<V4*>(d)[1] = y;
      }
    }
#pragma unroll
    for (int u = 0; u < B_PER; u++) {
      int g = t + u * 256;
      if (g < B_GROUPS) {
        int q = g % (BK / 4), n = g / (BK / 4);
        T* d0 = bs + ((2 * q) * BN + n) * 2;
        T* d1 = bs + ((2 * q + 1) * BN + n) * 2;
        d0[0] = rb[u].x; d0[1] = rb[u].y;
        d1[0] = rb[u].z; d1[1] = rb[u].w;
      }
    }
  };

  T acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; i++)
#pragma unroll
    for (int j = 0; j < TN; j++) acc[i][j] = Trop<T>::neg();

  const int nk = K / BK;
  gload(0);
  sstore(0);
  __syncthreads();
  for (int kt = 0; kt < nk; kt++) {
    const int buf = kt & 1;
    if (kt + 1 < nk) gload((kt + 1) * BK);
    const T* as = As + buf * Cfg::A_WORDS;
    const T* bs = Bs + buf * Cfg::B_WORDS;
#pragma unroll
    for (int kp = 0; kp < BK / 2; kp++) mp_step<T, TM, TN, BM, BN>(as, bs, kp, wm, wn, lm, ln, acc);
    if (kt + 1 < nk) {
      sstore(buf ^ 1);
    }
    __syncthreads();
  }
  // store
#pragma unroll
  for (int j = 0; j < TN; j++) {
    int n = n0 + gm_col<TN, BN>(wn, ln, j);
#pragma unroll
    for (int i = 0; i < TM; i++) {
      int m = m0 + gm_row<TM, BM>(wm, lm, i);
      Cb[(int64_t)n * M + m] = acc[i][j];
    }
  }
}

// ---------------------------------------------------------------------------
// fused GEMM tile: k-pair interleaved operands staged by bulk async copies
// ---------------------------------------------------------------------------
// Atomic max into the output of a split-K node.  int32: the integer max.
// f32: the int max of the bits, exact for values >= 0 and -inf (the only
// negative one, whose bits are a negative int): what MIS networks with
// weights >= 0 hold.  The output starts at kFillBits (STEP_FILL).
template <typename T>
__device__ __forceinline__ void red_max(T* p, T v) {
  if constexpr (std::is_same<T, float>::value) atomicMax(reinterpret_cast<int*>(p), __float_as_int(v));
  else atomicMax(reinterpret_cast<int*>(p), (int)v);
}

// STEP_FILL tile: kFillPerTile elements of a split-K node's output set to
// kFillBits (16-byte stores; the output is 32-element aligned).
template <typename T>
__device__ __forceinline__ void fill_tile(const GemmDesc& d, T* __restrict__ arena, int64_t tile) {
  const int64_t size = int64_t(1) << (d.m_log2 + d.n_log2 + d.bt_log2);
  int4* c = reinterpret_cast<int4*>(arena + d.c_fin);
  const int4 v = make_int4(kFillBits, kFillBits, kFillBits, kFillBits);
  for (int64_t q = tile * (kFillPerTile / 4) + threadIdx.x; q < (tile + 1) * (kFillPerTile / 4) && 4 * q < size;
       q += kThreads)
    c[q] = v;
}
constexpr int kGemmStages = 3;
constexpr int kGemmBK = 32;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, int count) {
  asm volatile("mbarrier.init.shared.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
  asm volatile("mbarrier.inval.shared.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait on one phase of an mbarrier: false when the limit is reached.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  for (int i = 0; i < (1 << 22); i++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

template <int BM, int BN, int S = kGemmStages, int BK = kGemmBK, bool I16 = false>
struct GemmSmem {
  static constexpr int KP = BK / 2;
  static constexpr int BAR_BYTES = 256;  // full[S] then empty[S] mbarriers (room for 16 stages)
  static constexpr int A_STAGE = KP * BM * 2;  // elements
  static constexpr int B_STAGE = KP * BN * 2;
  static constexpr int SCAT_OFF = BAR_BYTES + S * (A_STAGE + B_STAGE) * 4;  // epilogue tables
  static constexpr int PACK_OFF = SCAT_OFF + (BM + BN) * 4;  // two packed-int16 chunks (I16)
  static constexpr int PACK_WORDS = KP * (BM + BN);
  static constexpr int BYTES = PACK_OFF + (I16 ? 2 * PACK_WORDS * 4 : 0);
};

// Work units [u0, u1) of one GEMM descriptor on this CTA: unit u is output
// tile mn = u mod tiles_mn of batch point b and K part p (u / tiles_mn =
// p 2^bt + b).  The copies of every (unit, K chunk) of the run go through one
// ring of S stages, so the next unit's operands load while this unit's last
// chunks are reduced and its tile is stored.  Returns false after a timed-out
// wait (err is set; copies in flight are drained with a bounded wait).
// Copies of chunk q of a run (unit u0 + q / nkp, K chunk p nkp + q mod nkp)
// into stage `slot`; thread 0 only.  Everything is recomputed from the
// descriptor so none of it stays live in the consumers' registers.
template <typename T, int BM, int BN, int S, int BK>
__device__ __forceinline__ void gemm_issue(const GemmDesc& d, int64_t u0, int q, int slot, const T* arena,
                                           int* smem) {
  using SM = GemmSmem<BM, BN, S, BK>;
  constexpr int KP = SM::KP;
  constexpr int BK_LOG2 = BK == 32 ? 5 : 4;
  const int nkp_log2 = d.k_log2 - BK_LOG2 - d.ks_log2;
  const int tm_log2 = d.m_log2 - d.bm_log2, tmn_log2 = tm_log2 + d.n_log2 - d.bn_log2;
  const int64_t u = u0 + (q >> nkp_log2);
  const int64_t mn = u & ((int64_t(1) << tmn_log2) - 1), rest = u >> tmn_log2;
  const int64_t b = rest & ((int64_t(1) << d.bt_log2) - 1), part = rest >> d.bt_log2;
  const int m0 = (int)(mn & ((int64_t(1) << tm_log2) - 1)) * BM, n0 = (int)(mn >> tm_log2) * BN;
  const int64_t kc = (part << nkp_log2) + (q & ((1 << nkp_log2) - 1));
  const int64_t M = int64_t(1) << d.m_log2, N = int64_t(1) << d.n_log2, K = int64_t(1) << d.k_log2;
  const T* Ab = arena + d.a_off + b * M * K + 2 * m0;
  const T* Bb = arena + d.b_off + b * N * K + 2 * n0;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  T* As = reinterpret_cast<T*>(reinterpret_cast<char*>(smem) + SM::BAR_BYTES) + slot * SM::A_STAGE;
  T* Bs = reinterpret_cast<T*>(reinterpret_cast<char*>(smem) + SM::BAR_BYTES) + S * SM::A_STAGE + slot * SM::B_STAGE;
  mbar_expect_tx(&full[slot], (uint32_t)((SM::A_STAGE + SM::B_STAGE) * sizeof(T)));
  for (int kp = 0; kp < KP; kp++) {
    const int64_t row = kc * KP + kp;
    bulk_g2s(As + kp * BM * 2, Ab + row * 2 * M, BM * 2 * sizeof(T), &full[slot]);
    bulk_g2s(Bs + kp * BN * 2, Bb + row * 2 * N, BN * 2 * sizeof(T), &full[slot]);
  }
}

// Work units [u0, u1) of one GEMM descriptor on this CTA: unit u is output
// tile mn = u mod tiles_mn of batch point b and K part p (u / tiles_mn =
// p 2^bt + b).  The copies of every (unit, K chunk) of the run go through one
// ring of S stages, so the next unit's operands load while this unit's last
// chunks are reduced and its tile is stored.  Returns false after a timed-out
// wait (err is set; copies in flight are drained with a bounded wait).
template <typename T, int BM, int BN, int S = kGemmStages, int BK = kGemmBK, bool I16 = false>
__device__ bool gemm_tiles(const GemmDesc& d, int64_t u0, int64_t u1, T* __restrict__ arena, int* __restrict__ smem,
                           int* err, bool kpart_atomic = false) {
  using SM = GemmSmem<BM, BN, S, BK, I16>;
  using G = GemmShape<BM, BN>;
  constexpr int KP = SM::KP;
  constexpr int TM = G::TM, TN = G::TN;
  static_assert(!I16 || std::is_same<T, float>::value, "packed int16 tiles stand in for f32 values");
  using Acc = typename std::conditional<I16, uint32_t, T>::type;
  constexpr int BK_LOG2 = BK == 32 ? 5 : 4;
  static_assert(BK == 32 || BK == 16, "BK");
  const int t = threadIdx.x;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem);
  const T* As = reinterpret_cast<const T*>(reinterpret_cast<char*>(smem) + SM::BAR_BYTES);
  const T* Bs = As + S * SM::A_STAGE;
  int* scM = reinterpret_cast<int*>(reinterpret_cast<char*>(smem) + SM::SCAT_OFF);
  int* scN = scM + BM;
  const int nkp_log2 = d.k_log2 - BK_LOG2 - d.ks_log2;  // chunks of one unit
  const int n_units = (int)(u1 - u0);
  const int total_q = n_units << nkp_log2;
  // K = 16 (one chunk a unit, deep rings) with tiles of 64 x 64 or more: no
  // block barrier per chunk; each warp arrives on the stage's empty barrier
  // when done with it, and thread 0 refills the stage of the previous chunk
  // once all eight have (by then they usually have).  Measured on rr300w's
  // K = 16 levels: 128 x 128 tiles 1.88 -> 1.56 ms, but the skinny 256 x 16
  // tiles (shared-load bound) 2.98 -> 3.18 ms, so those keep the barrier.
  constexpr bool DEFER = BK == 16 && !I16 && BM >= 64 && BN >= 64;
  uint64_t* empty = full + 16;

  __syncthreads();  // the previous user of this shared memory is done
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  if (t == 0)
    for (int i = 0; i < S; i++) {
      mbar_init(&full[i], 1);
      if (DEFER) mbar_init(&empty[i], kThreads / 32);
    }
  // C offsets of the tile's rows / columns from their low bits: the scatter
  // is linear over disjoint bits, so a unit adds only its (m0, n0, b) base
  for (int i = t; i < BM; i += kThreads) {
    int o = 0;
    for (int x = 0; x < d.bm_log2; x++)
      if ((i >> x) & 1) o += 1 << d.m_pc[x];
    scM[i] = o;
  }
  for (int j = t; j < BN; j += kThreads) {
    int o = 0;
    for (int x = 0; x < d.bn_log2; x++)
      if ((j >> x) & 1) o += 1 << d.n_pc[x];
    scN[j] = o;
  }
  __syncthreads();
  int issued = 0;
  dep_wait();  // the arena's first access (the tables above read only the descriptor)
  if (t == 0)
    for (; issued < S && issued < total_q; issued++) gemm_issue<T, BM, BN, S, BK>(d, u0, issued, issued, arena, smem);

  // After a block barrier that ends a chunk, thread 0 refills its slot.  A
  // timed-out wait clears ok and the loops run on (results are discarded);
  // the failure is collected at the end.
  bool ok = true;
  int slot = 0;
  uint32_t par = 0;
  int q = 0;
  for (int ui = 0; ui < n_units; ui++) {
    const int warp = t >> 5, lane = t & 31;
    const int wm = G::wm(warp), wn = G::wn(warp), lm = G::lm(lane), ln = G::ln(lane);
    Acc acc[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; i++)
#pragma unroll
      for (int j = 0; j < TN; j++) {
        if constexpr (I16) acc[i][j] = 0x80008000u;  // below every sum
        else acc[i][j] = Trop<T>::neg();
      }
    for (int kl = 0; kl < (1 << nkp_log2); kl++, q++) {
      if (ok) ok = mbar_wait(&full[slot], par);
      const T* as = As + slot * SM::A_STAGE;
      const T* bs = Bs + slot * SM::B_STAGE;
      if constexpr (I16) {
        // the stage's f32 k-pairs become packed int16 words in one of two
        // chunk buffers (chunk q uses buffer q & 1: the last reader of that
        // buffer was chunk q - 2, which every thread finished before the
        // barrier of chunk q - 1)
        constexpr int NA = KP * BM, NB = KP * BN;
        uint32_t* pk =
            reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(smem) + SM::PACK_OFF) + (q & 1) * SM::PACK_WORDS;
        for (int e = t; e < NA; e += kThreads) {
          const float2 v = reinterpret_cast<const float2*>(as)[e];
          pk[e] = pack_i16(v.x, v.y);
        }
        for (int e = t; e < NB; e += kThreads) {
          const float2 v = reinterpret_cast<const float2*>(bs)[e];
          pk[NA + e] = pack_i16(v.x, v.y);
        }
        __syncthreads();  // the chunk's words are in place and its stage is free
        if (t == 0 && q + S < total_q && ok) {
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // reads above, then async writes
          gemm_issue<T, BM, BN, S, BK>(d, u0, q + S, slot, arena, smem);
          issued = q + S + 1;
        }
#pragma unroll 1
        for (int kp = 0; kp < KP; kp++) mp_step_i16<TM, TN, BM, BN>(pk, pk + NA, kp, wm, wn, lm, ln, acc);
      } else {
        // two k-pairs per iteration, so the next one's shared loads are issued
        // while this one's adds and maxes run
#pragma unroll 2
        for (int kp = 0; kp < KP; kp++) mp_step<T, TM, TN, BM, BN>(as, bs, kp, wm, wn, lm, ln, acc);
        if constexpr (DEFER) {
          __syncwarp();
          if (lane == 0) mbar_arrive(&empty[slot]);
          // chunk q - 1's stage takes chunk q - 1 + S
          const int pq = q - 1;
          if (t == 0 && pq >= 0 && pq + S < total_q && ok) {
            const int ps = slot == 0 ? S - 1 : slot - 1;
            ok = mbar_wait(&empty[ps], (uint32_t)((pq / S) & 1));
            if (ok) {
              asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // reads above, then async writes
              gemm_issue<T, BM, BN, S, BK>(d, u0, pq + S, ps, arena, smem);
              issued = pq + S + 1;
            }
          }
        } else {
          // every warp is done with this stage: thread 0 refills it at once (a
          // block barrier per chunk measured faster than per-warp arrivals on
          // an empty barrier that thread 0 waits on, with 32-wide chunks)
          __syncthreads();
          if (t == 0 && q + S < total_q && ok) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // reads above, then async writes
            gemm_issue<T, BM, BN, S, BK>(d, u0, q + S, slot, arena, smem);
            issued = q + S + 1;
          }
        }
      }
      if (++slot == S) {
        slot = 0;
        par ^= 1u;
      }
    }
    // epilogue: scatter the tile into C's layout (part p of a split K at
    // c_off + p 2^(m+n+bt), or by atomic max into the output c_fin)
    {
      const int tm_log2 = d.m_log2 - d.bm_log2, tmn_log2 = tm_log2 + d.n_log2 - d.bn_log2;
      const int64_t u = u0 + ui;
      const int64_t mn = u & ((int64_t(1) << tmn_log2) - 1), rest = u >> tmn_log2;
      const int64_t b = rest & ((int64_t(1) << d.bt_log2) - 1), part = rest >> d.bt_log2;
      const int mt = (int)(mn & ((int64_t(1) << tm_log2) - 1)), nt = (int)(mn >> tm_log2);
      const bool atomic = kpart_atomic && d.ks_log2 > 0;
      int64_t cb = atomic ? d.c_fin : d.c_off + (part << (d.m_log2 + d.n_log2 + d.bt_log2));
      for (int x = 0; x < d.bt_log2; x++)
        if ((b >> x) & 1) cb += int64_t(1) << d.b_pc[x];
      for (int x = d.bm_log2; x < d.m_log2; x++)
        if ((mt >> (x - d.bm_log2)) & 1) cb += int64_t(1) << d.m_pc[x];
      for (int x = d.bn_log2; x < d.n_log2; x++)
        if ((nt >> (x - d.bn_log2)) & 1) cb += int64_t(1) << d.n_pc[x];
      T* Cb = arena + cb;
      // rows i, i + 1 (i even) of a thread differ in m bit 0 when BM >= 64:
      // adjacent in C when m bit 0 sits at C position 0
      auto out = [&](int i, int j) -> T {
        if constexpr (I16) return unpack_max_i16(acc[i][j]);
        else return acc[i][j];
      };
      if (atomic) {
#pragma unroll
        for (int i = 0; i < TM; i++) {
          T* ro = Cb + scM[gm_row<TM, BM>(wm, lm, i)];
#pragma unroll
          for (int j = 0; j < TN; j++) red_max<T>(ro + scN[gm_col<TN, BN>(wn, ln, j)], out(i, j));
        }
      } else if (TM >= 4 && d.m_pc[0] == 0) {
#pragma unroll
        for (int i = 0; i < TM; i += 2) {
          T* ro = Cb + scM[gm_row<TM, BM>(wm, lm, i)];
#pragma unroll
          for (int j = 0; j < TN; j++) {
            typename Vec2<T>::type v;
            v.x = out(i, j);
            v.y = out(i + 1, j);
            *reinterpret_cast<typename Vec2<T>::type*>(ro + scN[gm_col<TN, BN>(wn, ln, j)]) = v;
          }
        }
      } else {
#pragma unroll
        for (int i = 0; i < TM; i++) {
          T* ro = Cb + scM[gm_row<TM, BM>(wm, lm, i)];
#pragma unroll
          for (int j = 0; j < TN; j++) ro[scN[gm_col<TN, BN>(wn, ln, j)]] = out(i, j);
        }
      }
    }
  }
  if (__syncthreads_or(!ok)) {
    if (t == 0) {
      atomicExch(err, 3 /* TB_ERR_TIMEOUT */);
      // a chunk before issued - S had its slot refilled only after thread 0
      // saw it land; the last S may still be in flight
      for (int j = issued > S ? issued - S : 0; j < issued; j++) mbar_wait(&full[j % S], (uint32_t)((j / S) & 1));
    }
    __syncthreads();
    return false;
  }
  // (the barrier of __syncthreads_or above: every warp's arrivals are in)
  if (t == 0)
    for (int i = 0; i < S; i++) {
      mbar_inval(&full[i]);
      if (DEFER) mbar_inval(&empty[i]);
    }
  return true;
}

template <typename T, int BM, int BN>
__device__ __forceinline__ bool gemm_tile(const GemmDesc& d, int64_t tile, T* arena, int* smem, int* err) {
  return gemm_tiles<T, BM, BN>(d, tile, tile + 1, arena, smem, err);
}

// Dispatch on the CTA tile shape chosen by the plan compiler.
template <typename T>
__device__ __forceinline__ bool gemm_tiles_any(const GemmDesc& d, int64_t u0, int64_t u1, T* arena, int* smem,
                                               int* err, bool i16 = false, bool kpart_atomic = false) {
  // copy stages: as many as fit the shared memory of the 128 x 128 form
  const int bm = d.bm_log2, bn = d.bn_log2;
  if (d.k_log2 < 5) {
    // K = 16: one 16-wide chunk a unit; the ring holds the next units' chunks
    if (bm == 7 && bn == 7) return gemm_tiles<T, 128, 128, 6, 16>(d, u0, u1, arena, smem, err, kpart_atomic);
    if (bm == 7 && bn == 6) return gemm_tiles<T, 128, 64, 8, 16>(d, u0, u1, arena, smem, err, kpart_atomic);
    if (bm == 6 && bn == 7) return gemm_tiles<T, 64, 128, 8, 16>(d, u0, u1, arena, smem, err, kpart_atomic);
    if (bm == 6 && bn == 6) return gemm_tiles<T, 64, 64, 12, 16>(d, u0, u1, arena, smem, err, kpart_atomic);
    if (bm == 8) return gemm_tiles<T, 256, 16, 5, 16>(d, u0, u1, arena, smem, err, kpart_atomic);
    if (bn == 8) return gemm_tiles<T, 16, 256, 5, 16>(d, u0, u1, arena, smem, err, kpart_atomic);
    if (bm >= 5 && bn >= 5) return gemm_tiles<T, 32, 32, 16, 16>(d, u0, u1, arena, smem, err, kpart_atomic);
    return gemm_tiles<T, 16, 16, 16, 16>(d, u0, u1, arena, smem, err, kpart_atomic);
  }
  if constexpr (std::is_same<T, float>::value) {
    // exact packed-int16 arithmetic for the large tiles (see pack_i16)
    if (i16) {
      if (bm == 7 && bn == 7) return gemm_tiles<T, 128, 128, 2, kGemmBK, true>(d, u0, u1, arena, smem, err, kpart_atomic);
      if (bm == 7 && bn == 6) return gemm_tiles<T, 128, 64, 3, kGemmBK, true>(d, u0, u1, arena, smem, err, kpart_atomic);
      if (bm == 6 && bn == 7) return gemm_tiles<T, 64, 128, 3, kGemmBK, true>(d, u0, u1, arena, smem, err, kpart_atomic);
    }
  }
  if (bm == 7 && bn == 7) return gemm_tiles<T, 128, 128, 3>(d, u0, u1, arena, smem, err, kpart_atomic);
  if (bm == 7 && bn == 6) return gemm_tiles<T, 128, 64, 4>(d, u0, u1, arena, smem, err, kpart_atomic);
  if (bm == 6 && bn == 7) return gemm_tiles<T, 64, 128, 4>(d, u0, u1, arena, smem, err, kpart_atomic);
  if (bm == 6 && bn == 6) return gemm_tiles<T, 64, 64, 6>(d, u0, u1, arena, smem, err, kpart_atomic);
  if (bm == 8) return gemm_tiles<T, 256, 16, 2>(d, u0, u1, arena, smem, err, kpart_atomic);
  if (bn == 8) return gemm_tiles<T, 16, 256, 2>(d, u0, u1, arena, smem, err, kpart_atomic);
  if (bm >= 5 && bn >= 5) return gemm_tiles<T, 32, 32, 8>(d, u0, u1, arena, smem, err, kpart_atomic);
  return gemm_tiles<T, 16, 16, 8>(d, u0, u1, arena, smem, err, kpart_atomic);
}
template <typename T>
__device__ __forceinline__ bool gemm_tile_any(const GemmDesc& d, int64_t tile, T* arena, int* smem, int* err) {
  return gemm_tiles_any<T>(d, tile, tile + 1, arena, smem, err);
}

__host__ __device__ constexpr int gemm_smem_bytes_max() { return GemmSmem<128, 128, 3>::BYTES; }
static_assert(GemmSmem<128, 128, 2, kGemmBK, true>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<128, 64, 3, kGemmBK, true>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<64, 128, 3, kGemmBK, true>::BYTES <= gemm_smem_bytes_max(),
              "packed-int16 GEMM stages exceed the shared memory of the 128 x 128 form");
static_assert(GemmSmem<128, 64, 4>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<64, 128, 4>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<64, 64, 6>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<32, 32, 8>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<16, 16, 8>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<256, 16, 2>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<16, 256, 2>::BYTES <= gemm_smem_bytes_max(),
              "GEMM stages exceed the shared memory of the 128 x 128 form");
static_assert(GemmSmem<128, 128, 6, 16>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<128, 64, 8, 16>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<64, 128, 8, 16>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<64, 64, 12, 16>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<32, 32, 16, 16>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<16, 16, 16, 16>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<256, 16, 5, 16>::BYTES <= gemm_smem_bytes_max() &&
                  GemmSmem<16, 256, 5, 16>::BYTES <= gemm_smem_bytes_max(),
              "K=16 GEMM stages exceed the shared memory of the 128 x 128 form");
static_assert(2 * 16 * 8 <= GemmSmem<16, 16>::BAR_BYTES, "full and empty mbarriers of 16 stages");
static_assert(gm_covers<128, 128>() && gm_covers<128, 64>() && gm_covers<64, 128>() && gm_covers<64, 64>() &&
                  gm_covers<32, 32>() && gm_covers<16, 16>() && gm_covers<256, 16>() && gm_covers<16, 256>(),
              "GEMM tile thread layouts");

}  // namespace tb
