// Semiring arithmetic with Julia Base semantics, shared by the SpMV/SpMM
// kernels.  Integers wrap (two's complement, like Julia's Int32/Int64 `+`
// and `*`); float min/max follow Julia's @fastmath min_fast/max_fast, which
// Finch's generated code runs under (src/execute.jl:116-120): the second
// operand wins only when strictly smaller (larger).  Identities follow
// Finch's algebra traits (src/symbolic/symbolic.jl:95-104).
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include <cfloat>
#include <climits>

namespace fgb {

enum { SR_PT = 0, SR_MINP = 1, SR_MAXP = 2, SR_OA = 3 };
enum { FM_DEFAULT = 0, FM_FMA = 1, FM_NOFMA = 2 };

// ---- stored value -> accumulation type
template <class A, class V>
__device__ __forceinline__ A to_acc(V v) {
  return (A)v;
}
template <>
__device__ __forceinline__ float to_acc<float, __nv_bfloat16>(__nv_bfloat16 v) {
  return __bfloat162float(v);
}

// ---- wrapping integer arithmetic
__device__ __forceinline__ int32_t wadd(int32_t a, int32_t b) {
  return (int32_t)((uint32_t)a + (uint32_t)b);
}
__device__ __forceinline__ int64_t wadd(int64_t a, int64_t b) {
  return (int64_t)((uint64_t)a + (uint64_t)b);
}
__device__ __forceinline__ int32_t wmul(int32_t a, int32_t b) {
  return (int32_t)((uint32_t)a * (uint32_t)b);
}
__device__ __forceinline__ int64_t wmul(int64_t a, int64_t b) {
  return (int64_t)((uint64_t)a * (uint64_t)b);
}
__device__ __forceinline__ double wadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float wadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double wmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float wmul(float a, float b) { return __fmul_rn(a, b); }

__device__ __forceinline__ double fused(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float fused(float a, float b, float c) { return __fmaf_rn(a, b, c); }

template <class A>
struct Lim;
template <>
struct Lim<double> {
  __device__ static double hi() { return __longlong_as_double(0x7ff0000000000000LL); }
  __device__ static double lo() { return __longlong_as_double((long long)0xfff0000000000000ULL); }
};
template <>
struct Lim<float> {
  __device__ static float hi() { return __int_as_float(0x7f800000); }
  __device__ static float lo() { return __int_as_float((int)0xff800000u); }
};
template <>
struct Lim<int32_t> {
  __device__ static int32_t hi() { return INT32_MAX; }
  __device__ static int32_t lo() { return INT32_MIN; }
};
template <>
struct Lim<int64_t> {
  __device__ static int64_t hi() { return INT64_MAX; }
  __device__ static int64_t lo() { return INT64_MIN; }
};

template <class A>
__device__ __forceinline__ A jmin(A a, A b) {
  return (b < a) ? b : a;
}
template <class A>
__device__ __forceinline__ A jmax(A a, A b) {
  return (b > a) ? b : a;
}

template <int SR, class A>
struct Semi;

template <class A>
struct Semi<SR_PT, A> {
  __device__ static A identity() { return (A)0; }
  __device__ static A one() { return (A)1; }
  __device__ static A add(A acc, A t) { return wadd(acc, t); }
  __device__ static A mul(A a, A x) { return wmul(x, a); }
  // acc <- acc (+) a (*) x  with the requested contraction for floats.
  __device__ static A step(A acc, A a, A x, int fm) { return wadd(wmul(x, a), acc); }
};
template <>
struct Semi<SR_PT, double> {
  __device__ static double identity() { return 0.0; }
  __device__ static double one() { return 1.0; }
  __device__ static double add(double acc, double t) { return __dadd_rn(acc, t); }
  __device__ static double mul(double a, double x) { return __dmul_rn(x, a); }
  __device__ static double step(double acc, double a, double x, int fm) {
    return fm == FM_NOFMA ? __dadd_rn(__dmul_rn(x, a), acc) : __fma_rn(x, a, acc);
  }
};
template <>
struct Semi<SR_PT, float> {
  __device__ static float identity() { return 0.f; }
  __device__ static float one() { return 1.f; }
  __device__ static float add(float acc, float t) { return __fadd_rn(acc, t); }
  __device__ static float mul(float a, float x) { return __fmul_rn(x, a); }
  __device__ static float step(float acc, float a, float x, int fm) {
    return fm == FM_NOFMA ? __fadd_rn(__fmul_rn(x, a), acc) : __fmaf_rn(x, a, acc);
  }
};

template <class A>
struct Semi<SR_MINP, A> {
  __device__ static A identity() { return Lim<A>::hi(); }
  __device__ static A one() { return (A)0; }
  __device__ static A add(A acc, A t) { return jmin(acc, t); }
  __device__ static A mul(A a, A x) { return wadd(a, x); }
  __device__ static A step(A acc, A a, A x, int) { return jmin(acc, wadd(a, x)); }
};

template <class A>
struct Semi<SR_MAXP, A> {
  __device__ static A identity() { return Lim<A>::lo(); }
  __device__ static A one() { return (A)0; }
  __device__ static A add(A acc, A t) { return jmax(acc, t); }
  __device__ static A mul(A a, A x) { return wadd(a, x); }
  __device__ static A step(A acc, A a, A x, int) { return jmax(acc, wadd(a, x)); }
};

template <>
struct Semi<SR_OA, uint8_t> {
  __device__ static uint8_t identity() { return 0; }
  __device__ static uint8_t one() { return 1; }
  __device__ static uint8_t add(uint8_t acc, uint8_t t) { return acc | t; }
  __device__ static uint8_t mul(uint8_t a, uint8_t x) { return a & x; }
  __device__ static uint8_t step(uint8_t acc, uint8_t a, uint8_t x, int) { return acc | (a & x); }
};

// ---- lane shuffles for every accumulation type
// Mask of the G-lane group (G a power of two <= 32) that owns this lane.
template <int G>
__device__ __forceinline__ unsigned group_mask() {
  return G == 32 ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
}

template <class A>
__device__ __forceinline__ A shfl_xor(unsigned mask, A v, int m, int width) {
  return __shfl_xor_sync(mask, v, m, width);
}
template <>
__device__ __forceinline__ uint8_t shfl_xor<uint8_t>(unsigned mask, uint8_t v, int m, int width) {
  return (uint8_t)__shfl_xor_sync(mask, (int)v, m, width);
}

// ---- atomic (+)-updates for push kernels
template <int SR, class A>
struct AtomicAdd;

template <>
struct AtomicAdd<SR_PT, double> {
  __device__ static void apply(double* p, double t) { atomicAdd(p, t); }
};
template <>
struct AtomicAdd<SR_PT, float> {
  __device__ static void apply(float* p, float t) { atomicAdd(p, t); }
};
template <>
struct AtomicAdd<SR_PT, int32_t> {
  __device__ static void apply(int32_t* p, int32_t t) { atomicAdd((int*)p, (int)t); }
};
template <>
struct AtomicAdd<SR_PT, int64_t> {
  __device__ static void apply(int64_t* p, int64_t t) {
    atomicAdd((unsigned long long*)p, (unsigned long long)t);
  }
};
template <>
struct AtomicAdd<SR_MINP, int32_t> {
  __device__ static void apply(int32_t* p, int32_t t) {
    if (t < *(volatile int32_t*)p) atomicMin((int*)p, (int)t);
  }
};
template <>
struct AtomicAdd<SR_MINP, int64_t> {
  __device__ static void apply(int64_t* p, int64_t t) {
    if (t < *(volatile int64_t*)p) atomicMin((long long*)p, (long long)t);
  }
};
template <>
struct AtomicAdd<SR_MAXP, int32_t> {
  __device__ static void apply(int32_t* p, int32_t t) {
    if (t > *(volatile int32_t*)p) atomicMax((int*)p, (int)t);
  }
};
template <>
struct AtomicAdd<SR_MAXP, int64_t> {
  __device__ static void apply(int64_t* p, int64_t t) {
    if (t > *(volatile int64_t*)p) atomicMax((long long*)p, (long long)t);
  }
};
// Float min/max through compare-and-swap on the bit pattern.  Values only
// move in one direction, so a stale read that already beats `t` ends the loop.
template <>
struct AtomicAdd<SR_MINP, double> {
  __device__ static void apply(double* p, double t) {
    unsigned long long* a = (unsigned long long*)p;
    unsigned long long old = *(volatile unsigned long long*)a;
    while (t < __longlong_as_double((long long)old)) {
      unsigned long long prev = atomicCAS(a, old, (unsigned long long)__double_as_longlong(t));
      if (prev == old) break;
      old = prev;
    }
  }
};
template <>
struct AtomicAdd<SR_MINP, float> {
  __device__ static void apply(float* p, float t) {
    unsigned* a = (unsigned*)p;
    unsigned old = *(volatile unsigned*)a;
    while (t < __uint_as_float(old)) {
      unsigned prev = atomicCAS(a, old, __float_as_uint(t));
      if (prev == old) break;
      old = prev;
    }
  }
};
template <>
struct AtomicAdd<SR_MAXP, double> {
  __device__ static void apply(double* p, double t) {
    unsigned long long* a = (unsigned long long*)p;
    unsigned long long old = *(volatile unsigned long long*)a;
    while (t > __longlong_as_double((long long)old)) {
      unsigned long long prev = atomicCAS(a, old, (unsigned long long)__double_as_longlong(t));
      if (prev == old) break;
      old = prev;
    }
  }
};
template <>
struct AtomicAdd<SR_MAXP, float> {
  __device__ static void apply(float* p, float t) {
    unsigned* a = (unsigned*)p;
    unsigned old = *(volatile unsigned*)a;
    while (t > __uint_as_float(old)) {
      unsigned prev = atomicCAS(a, old, __float_as_uint(t));
      if (prev == old) break;
      old = prev;
    }
  }
};
// y |= t on a Bool byte: idempotent, so a plain store of `true` is exact.
template <>
struct AtomicAdd<SR_OA, uint8_t> {
  __device__ static void apply(uint8_t* p, uint8_t t) {
    if (t) *(volatile uint8_t*)p = 1;
  }
};

}  // namespace fgb
