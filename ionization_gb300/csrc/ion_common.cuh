// Shared device/host helpers for the ionization_gb300 CUDA library (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ionization_gb300.h"

namespace ion {

// ---------------------------------------------------------------------------
// complex numbers over a real type R (double for c128, float for c64)
// ---------------------------------------------------------------------------
template <typename R>
struct Cx {
    R re, im;
};

template <typename R> struct Vec2;
template <> struct Vec2<double> { using type = double2; };
template <> struct Vec2<float> { using type = float2; };

template <typename R>
__device__ __forceinline__ Cx<R> cx(R re, R im) { return Cx<R>{re, im}; }

template <typename R>
__device__ __forceinline__ Cx<R> operator+(Cx<R> a, Cx<R> b) { return {a.re + b.re, a.im + b.im}; }
template <typename R>
__device__ __forceinline__ Cx<R> operator-(Cx<R> a, Cx<R> b) { return {a.re - b.re, a.im - b.im}; }
template <typename R>
__device__ __forceinline__ Cx<R> operator-(Cx<R> a) { return {-a.re, -a.im}; }
template <typename R>
__device__ __forceinline__ Cx<R> operator*(Cx<R> a, Cx<R> b) {
    return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
template <typename R>
__device__ __forceinline__ Cx<R> scale(Cx<R> a, R s) { return {a.re * s, a.im * s}; }
// i * h * a for real h: (-h a.im, h a.re)
template <typename R>
__device__ __forceinline__ Cx<R> mul_ih(R h, Cx<R> a) { return {-h * a.im, h * a.re}; }

// 1/z as conj(z)/|z|^2.  The scalar division is the compiler's IEEE division.
template <typename R>
__device__ __forceinline__ Cx<R> crecip(Cx<R> z) {
    R inv = R(1) / (z.re * z.re + z.im * z.im);
    return {z.re * inv, -z.im * inv};
}

template <typename R>
__device__ __forceinline__ Cx<R> ld(const Cx<R>* p) {
    typename Vec2<R>::type v = *reinterpret_cast<const typename Vec2<R>::type*>(p);
    return {v.x, v.y};
}
template <typename R>
__device__ __forceinline__ void st(Cx<R>* p, Cx<R> a) {
    typename Vec2<R>::type v;
    v.x = a.re;
    v.y = a.im;
    *reinterpret_cast<typename Vec2<R>::type*>(p) = v;
}

// ---------------------------------------------------------------------------
// The stored residual of a complex64 state with residual (c64x): psi = g + lo
// with g complex64 and lo two bf16 in one 32-bit word (re in the low half,
// im in the high half), 12 bytes per point.  |lo| <= ulp(g) / 2 after every
// renormalisation, so its 8 significant bits carry psi to ~33 bits; bf16
// keeps FP32's exponent range, so lo needs no scaling.  Packing rounds each
// component to nearest even (cvt.rn.bf16x2.f32); unpacking is exact.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t lo_pack(Cx<float> v) {
    uint32_t w;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(w) : "f"(v.im), "f"(v.re));
    return w;
}
__device__ __forceinline__ Cx<float> lo_unpack(uint32_t w) {
    return Cx<float>{__uint_as_float(w << 16), __uint_as_float(w & 0xffff0000u)};
}
// lo as a later unpack of its packed form sees it
__device__ __forceinline__ Cx<float> lo_round(Cx<float> v) { return lo_unpack(lo_pack(v)); }

// ---------------------------------------------------------------------------
// host-side status plumbing
// ---------------------------------------------------------------------------
void set_error(const char* fmt, ...);
const char* last_error();
int check_launch(const char* what);
// the current device and the id of its current context (ion_runtime.cu)
int current_context(int* dev, unsigned long long* ctx_id);
// raise `kernel`'s dynamic shared-memory limit to `bytes` in the current
// context, once per (kernel, device, context); ION_OK or ION_ERR_CUDA
int ensure_smem_limit(const void* kernel, int bytes, const char* name);

// Streams and events for running independent launches side by side: fork
// with an event recorded on the caller's stream, join by making it wait for
// an event recorded on each side stream (also inside stream capture, where
// these become graph edges).  Made once per caller stream, device and
// context, outside capture: a stream whose first call is made under capture
// gets NULL and runs in stream order, as does any call when they cannot be
// made.
struct ForkJoin {
    static constexpr int N = 7;
    cudaStream_t s[N];
    cudaEvent_t fork;
    cudaEvent_t join[N];
};
ForkJoin* fork_join(cudaStream_t main);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// multiprocessors of the current device (queried once per device)
inline int num_sms() {
    static int cached[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 152;
    if (cached[dev] == 0) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cached[dev] = n > 0 ? n : 152;
    }
    return cached[dev];
}

}  // namespace ion
