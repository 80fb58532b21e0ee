// tmc_device.cuh — device building blocks of the photon walk (sm_103a).
//
// Reference: computacionparalela/tiny_mc photon.c:6-51 (one photon per call,
// global libc rand()).  Here one thread carries one photon at a time; the
// random numbers come from a Philox-4x32-10 stream keyed by the photon id, so
// the walk of photon p is the same whichever thread, warp or launch runs it.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "tmc.h"

namespace tmc {

constexpr unsigned FULL_MASK = 0xffffffffu;

// ----------------------------------------------------------------- Philox
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).  The ten round keys
// depend only on the seed, so they are precomputed on the host and passed in
// the kernel parameter block: every XOR with a key then reads the constant
// bank instead of spending an add per round.
constexpr uint32_t PHILOX_M0 = 0xD2511F53u;
constexpr uint32_t PHILOX_M1 = 0xCD9E8D57u;
constexpr uint32_t PHILOX_W0 = 0x9E3779B9u;
constexpr uint32_t PHILOX_W1 = 0xBB67AE85u;

struct PhiloxKeys {
    uint32_t k0[10];
    uint32_t k1[10];
};

inline PhiloxKeys make_philox_keys(uint64_t seed)
{
    PhiloxKeys k;
    uint32_t a = (uint32_t)seed, b = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; ++r) {
        k.k0[r] = a;
        k.k1[r] = b;
        a += PHILOX_W0;
        b += PHILOX_W1;
    }
    return k;
}

// Counter {c0, c1, c2, c3} -> four 32-bit words.
__device__ __forceinline__ uint4 philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                               const PhiloxKeys &K)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const unsigned long long p0 = (unsigned long long)PHILOX_M0 * c0;
        const unsigned long long p1 = (unsigned long long)PHILOX_M1 * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ K.k0[r];
        const uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ K.k1[r];
        c1 = (uint32_t)p1;
        c3 = (uint32_t)p0;
        c0 = n0;
        c2 = n2;
    }
    return make_uint4(c0, c1, c2, c3);
}

// rand() of photon.c: 31 bits of a Philox word; 0 becomes 1 so that
// -log(rand()/RAND_MAX) is always finite (the reference's logf(0) case).
__device__ __forceinline__ uint32_t rand31(uint32_t word)
{
    return max(word >> 1, 1u);
}

// rand()/(float)RAND_MAX: (float)RAND_MAX is exactly 2^31, so the quotient is
// the correctly rounded int->float conversion scaled by 2^-31 (exact).
__device__ __forceinline__ float uniform01(uint32_t word)
{
    return __uint2float_rn(rand31(word)) * 0x1p-31f;
}

// 2.0f*rand()/(float)RAND_MAX - 1.0f: 2*fl(r)/2^31 is exact, so one fused
// multiply-add rounds exactly once where photon.c rounds once (the "- 1").
// rand31's 0 -> 1 mapping is left out here because it cannot change the
// result: -1 + 2^-30 rounds to -1.0f (the float spacing next to -1 is 2^-24),
// the same value r = 0 gives.
__device__ __forceinline__ float uniform_pm1(uint32_t word)
{
    return fmaf(__uint2float_rn(word >> 1), 0x1p-30f, -1.0f);
}

// ------------------------------------------------------------ arithmetic
// The library's logarithm for TMC_MATH_EXACT, division-free: x = 2^k m with
// m in [sqrt(1/2), sqrt(2)), f = m - 1 (exact), log(m) = f + f^2 R(f) with R
// a degree-8 polynomial (the Chebyshev interpolant of log1p(f)/f at 10 nodes
// on [sqrt(1/2)-1, sqrt(2)-1], coefficients rounded to float; oracle/logfit.py
// derives them), evaluated by Horner with fused multiply-adds, and log x =
// k ln2_hi + (k ln2_lo + log m) with ln2 split so k ln2_hi is exact.  Every
// step is one IEEE-rounded operation (fma rounds once), so the CPU
// restatement reproduces it bit for bit.  Max error 0.86 ulp over every float
// in [2^-31, 1] (98.3% correctly rounded).
__device__ __forceinline__ float log_exact(float x)
{
    const uint32_t ix = __float_as_uint(x);
    const int k = (int)((ix + 0x004afb0du) >> 23) - 127;
    const float m = __uint_as_float(ix - ((uint32_t)k << 23));
    const float f = __fsub_rn(m, 1.0f);
    const float f2 = __fmul_rn(f, f);
    float r = -0x1.31335ap-4f;
    r = __fmaf_rn(r, f, 0x1.064786p-3f);
    r = __fmaf_rn(r, f, -0x1.0fb036p-3f);
    r = __fmaf_rn(r, f, 0x1.22cf10p-3f);
    r = __fmaf_rn(r, f, -0x1.5423b0p-3f);
    r = __fmaf_rn(r, f, 0x1.999e86p-3f);
    r = __fmaf_rn(r, f, -0x1.000424p-2f);
    r = __fmaf_rn(r, f, 0x1.55555ep-2f);
    r = __fmaf_rn(r, f, -0x1.fffff8p-2f);
    const float lm = __fmaf_rn(f2, r, f);
    const float kf = __int2float_rn(k);
    return __fmaf_rn(kf, 0.693145751953125f, __fmaf_rn(kf, 1.42860682e-6f, lm));
}

__device__ __forceinline__ float sqrt_approx(float x)
{
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// photon.c's float expressions, IEEE-rounded one operation at a time.
struct ExactMath {
    static constexpr uint32_t id = TMC_MATH_EXACT;
    // -logf(U), photon.c:21
    __device__ static __forceinline__ float step_length(float U) { return -log_exact(U); }
    // x += t * u, photon.c:22-24
    __device__ static __forceinline__ float move(float x, float t, float u)
    {
        return __fadd_rn(x, __fmul_rn(t, u));
    }
    // sqrtf(x*x + y*y + z*z) * shells_per_mfp, photon.c:26
    __device__ static __forceinline__ float radius_shells(float x, float y, float z, float spm)
    {
        const float r2 = __fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z));
        return __fmul_rn(__fsqrt_rn(r2), spm);
    }
    // xi1*xi1 + xi2*xi2, photon.c:39
    __device__ static __forceinline__ float norm2(float a, float b)
    {
        return __fadd_rn(__fmul_rn(a, a), __fmul_rn(b, b));
    }
    // sqrtf((1.0f - u*u) / t), photon.c:42-43
    __device__ static __forceinline__ float dir_scale(float t, float u)
    {
        return __fsqrt_rn(__fdiv_rn(__fsub_rn(1.0f, __fmul_rn(u, u)), t));
    }
    __device__ static __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
};

// Hardware approximations (MUFU lg2 / sqrt), contraction allowed.
struct FastMath {
    static constexpr uint32_t id = TMC_MATH_FAST;
    __device__ static __forceinline__ float step_length(float U) { return -__logf(U); }
    __device__ static __forceinline__ float move(float x, float t, float u) { return fmaf(t, u, x); }
    __device__ static __forceinline__ float radius_shells(float x, float y, float z, float spm)
    {
        return sqrt_approx(fmaf(x, x, fmaf(y, y, z * z))) * spm;
    }
    __device__ static __forceinline__ float norm2(float a, float b) { return fmaf(a, a, b * b); }
    // (1-u^2)/t with u = 2t-1 is 4(1-t): sqrt of it is 2 sqrt(1-t)
    __device__ static __forceinline__ float dir_scale(float t, float)
    {
        return 2.0f * sqrt_approx(1.0f - t);
    }
    __device__ static __forceinline__ float mul(float a, float b) { return a * b; }
};

// ---------------------------------------------------------------- tallies
// Fixed point of a deposit weight: rint(w * 2^40), returned as 32-bit halves,
// for 0 <= w <= 1 (a deposit is at most 2^40 units).  hi = floor(w * 2^8);
// the remainder w*2^40 - hi*2^32 is exact in one fused multiply-add (it is
// the low part of w's own significand), and its correctly rounded conversion
// is the low word: exact for w >= 2^-17, where w*2^40 is an integer, and
// round-to-nearest-even below.  No branch, and no float->u64 conversion (that
// one runs on the FP64 pipe).
__device__ __forceinline__ void fx40_split(float w, uint32_t &lo, uint32_t &hi)
{
    hi = __float2uint_rz(w * 0x1p8f);
    const float rem = fmaf(-__uint2float_rn(hi), 0x1p32f, w * 0x1p40f);
    lo = __float2uint_rn(rem);
}

// Add (hi:lo) to a 64-bit shared-memory tally kept as two 32-bit words, with
// native 32-bit shared atomics: the carry out of the low word goes into the
// high word, and a wrap of the high word carries 2^64 units into the 128-bit
// global tally.  The global word receives only such carries until the final
// flush, so no epoch barriers are needed however many photons a block walks.
// wraps (may be null) additionally counts this tally's 2^64 wraps.
__device__ __forceinline__ void tally_add(uint32_t *sh_lo, uint32_t *sh_hi,
                                          unsigned long long *g_hi, uint32_t lo, uint32_t hi,
                                          uint32_t *wraps = nullptr)
{
    const uint32_t old = atomicAdd(sh_lo, lo);
    hi += (old + lo < old) ? 1u : 0u;
    const uint32_t oh = atomicAdd(sh_hi, hi);
    if (oh + hi < oh) {
        atomicAdd(g_hi, 1ull);
        if (wraps)
            atomicAdd(wraps, 1u);
    }
}

// tally_add for a 64-bit sum that cannot wrap (the caller bounds it): the
// low word's carry goes into the high word, whose old value is not needed.
__device__ __forceinline__ void tally_add_nowrap(uint32_t *sh_lo, uint32_t *sh_hi, uint32_t lo, uint32_t hi)
{
    const uint32_t old = atomicAdd(sh_lo, lo);
    hi += (old + lo < old) ? 1u : 0u;
    atomicAdd(sh_hi, hi);
}

// Flush a 64-bit partial sum into a 128-bit global tally.
__device__ __forceinline__ void flush128(unsigned long long *g_lo, unsigned long long *g_hi,
                                         unsigned long long v)
{
    if (v) {
        const unsigned long long old = atomicAdd(g_lo, v);
        if (old + v < old)
            atomicAdd(g_hi, 1ull);
    }
}

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(FULL_MASK, v, o);
    return v;
}

}  // namespace tmc
