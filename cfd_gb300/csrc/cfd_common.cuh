// cfd_common.cuh — shared definitions of the cfd_gb300 CUDA library (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>

#include "../../include/cfd_gpu.h"

namespace cfd {

// ------------------------------------------------------------------ error plumbing
extern std::atomic<long long> g_launches;

#define CFD_CUDA(call)                                                          \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess) {                                                \
            cfd::set_last_cuda_error(e_, #call, __FILE__, __LINE__);            \
            return e_ == cudaErrorMemoryAllocation ? CFD_ERR_NOMEM : CFD_ERR_CUDA; \
        }                                                                       \
    } while (0)

// launch + count + check the launch error
#define CFD_LAUNCH(kernel, grid, block, smem, stream, ...)                      \
    do {                                                                        \
        kernel<<<(grid), (block), (smem), (stream)>>>(__VA_ARGS__);             \
        cfd::g_launches.fetch_add(1, std::memory_order_relaxed);                \
        CFD_CUDA(cudaGetLastError());                                           \
    } while (0)

void set_last_cuda_error(cudaError_t e, const char* what, const char* file, int line);

inline unsigned blocks_for(long n, int threads) {
    long b = (n + threads - 1) / threads;
    return (unsigned)(b > 0 ? b : 1);
}

// ------------------------------------------------------------------ x / 3 in three FP64 ops
// The correctly rounded quotient x / 3.0 (what the IEEE division returns) from a multiply
// and two FMAs.  R3 = RN(1/3) = (1/3)(1 - 2^-54), so q0 = RN(x * R3) is within one ulp of
// x/3 (|x*R3 - x/3| = |x/3| 2^-54 < ulp(x/3)/2, plus the product's rounding below ulp/2);
// then the remainder r = x - 3*q0 is exact in one FMA and RN(q0 + r*R3) is the correctly
// rounded x/3 (P. Markstein, IBM J. Res. Dev. 34(1), 1990; the divisor-known-in-advance
// form of N. Brisebarre, J.-M. Muller, S. K. Raina, IEEE Trans. Computers 53(8), 2004).
// The exponent check keeps every intermediate normal and finite; zeros, subnormals, huge
// values, infinities and NaNs take the plain division.  Bit-identical to x / 3.0 for every
// input (checked on the GPU against the division over random and edge-case inputs).
__device__ __forceinline__ double div3(double x) {
    const unsigned hi = (unsigned)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ffu;
    if (hi - 64u > 1936u) return x / 3.0;  // biased exponent outside [64, 2000]
    constexpr double R3 = 0x1.5555555555555p-2;
    const double q0 = x * R3;
    const double r = fma(-3.0, q0, x);
    return fma(r, R3, q0);
}

// x / d correctly rounded from y = RN(1/d) (formed once per d, by the division) in a
// multiply and four FMAs: q0 = RN(x*y) is within 1.5 ulp of x/d; one correction
// q1 = RN(q0 + RN(x - d*q0)*y) brings it within an ulp (the remainder's rounding and the
// product error move it by far less than an ulp); with q1 within an ulp the remainder
// x - d*q1 is exact in one FMA and RN(q1 + (x - d*q1)*y) is the correctly rounded x/d
// (Markstein's theorem: y within half an ulp of 1/d, q1 within an ulp of x/d).  The range
// check (both exponents and the quotient's) keeps every intermediate normal and finite;
// other operands (zeros included) take the division.  Bit-identical to x / d (checked on the GPU against the division).
__device__ __forceinline__ double div_rcp(double x, double d, double y) {
    const int ex = (int)((unsigned long long)__double_as_longlong(x) >> 52) & 0x7ff;
    const int ed = (int)((unsigned long long)__double_as_longlong(d) >> 52) & 0x7ff;
    // both exponents in [200, 1800] and the quotient's within 2^+-800
    if ((unsigned)(ex - 200) > 1600u || (unsigned)(ed - 200) > 1600u || abs(ex - ed) > 800)
        return x / d;
    const double q0 = x * y;
    const double q1 = fma(fma(-d, q0, x), y, q0);
    return fma(fma(-d, q1, x), y, q1);
}

// ------------------------------------------------------------------ FP32 <-> FP64 by bits
// GB300's FP64 pipe (1/64 of the FP32 rate) also executes the F2F conversions, so the
// mixed-precision kernels move values between the two formats with integer operations.
//   f2d_bits:  exact for normal floats, zeros, infinities and NaNs; a subnormal float (below
//              1.2e-38) becomes a zero of the same sign.
//   d2f_trunc: the significand truncated to 24 bits (error below 1 ulp of the float);
//              magnitudes below the float normal range give a signed zero, above it an
//              infinity.
//   split_bits: hi = d2f_trunc(v), lo = d2f_trunc(v - hi); the subtraction is exact, and
//              hi + lo equals v to within 2^-47 |v|.
__device__ __forceinline__ double f2d_bits(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned e = (u >> 23) & 0xffu;
    const unsigned long long sign = (unsigned long long)(u >> 31) << 63;
    const unsigned long long frac = (unsigned long long)(u & 0x7fffffu) << 29;
    if (e == 0u) return __longlong_as_double((long long)sign);
    const unsigned long long ex = (e == 0xffu) ? 0x7ffull : (unsigned long long)(e + 896u);
    return __longlong_as_double((long long)(sign | (ex << 52) | frac));
}

__device__ __forceinline__ float d2f_trunc(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const int e = (int)((b >> 52) & 0x7ffull);
    const unsigned frac = (unsigned)((b >> 29) & 0x7fffffull);
    if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | (frac ? 0x400000u : 0u));
    const int fe = e - 896;
    if (fe <= 0) return __uint_as_float(sign);
    if (fe >= 0xff) return __uint_as_float(sign | 0x7f800000u);
    return __uint_as_float(sign | ((unsigned)fe << 23) | frac);
}

// lo is formed from the bits as well: v - hd (hd = v with the low 29 significand bits
// cleared) is exactly m * 2^(e - 1075), m those 29 bits, so its float truncation takes the
// 24 bits from m's leading one; m = 0 gives +0 (as the FP64 difference v - v does).  Only
// infinities and NaNs take the FP64 subtraction.
__device__ __forceinline__ void split_bits(double v, float& hi, float& lo) {
    hi = d2f_trunc(v);
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const int e = (int)((b >> 52) & 0x7ffull);
    if (e == 0x7ff) {
        const double hd = __longlong_as_double((long long)(b & ~0x1fffffffull));
        lo = d2f_trunc(v - hd);
        return;
    }
    const unsigned m = (unsigned)(b & 0x1fffffffull);
    if (m == 0u) {
        lo = 0.f;
        return;
    }
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const int k = 31 - __clz((int)m);  // leading one of m
    const int fe = k + e - 948;        // the float exponent field of m * 2^(e - 1075)
    if (fe <= 0) {
        lo = __uint_as_float(sign);
    } else if (fe >= 0xff) {
        lo = __uint_as_float(sign | 0x7f800000u);
    } else {
        const unsigned mant = (k >= 23 ? (m >> (k - 23)) : (m << (23 - k))) & 0x7fffffu;
        lo = __uint_as_float(sign | ((unsigned)fe << 23) | mant);
    }
}

// ------------------------------------------------------------------ fixed-order sums
// The dot-product order every FP64 reduction of this library takes (and the oracle's
// or_vecdot restates): chunks of 1024 terms, lane t of a 256-thread block sums terms
// t, t+256, t+512, t+768 in that order; a shuffle-down tree over each warp's 32 lanes;
// an 8-way shuffle-down tree over the warps.  Chunk partials are folded by 256 lanes
// with stride 256, then the same 256-lane tree.
constexpr int kChunk = 1024;
constexpr int kRedThreads = 256;

__device__ __forceinline__ double warp_tree32(double v) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) v = v + __shfl_down_sync(0xffffffffu, v, off);
    return v;  // lane 0
}

// 256-lane tree; every thread of the block gets the result.  `red` holds >= 9 doubles.
// The tree: within each warp w of values v[32w .. 32w+31], the shuffle-down pairs
// (l, l+16), (l, l+8), (l, l+4), (l, l+2), (l, l+1); across the eight warp sums (w, w+4),
// (w, w+2), (w, w+1).  The same sums are formed by warp 0 alone: lane 4w+l (l < 4) adds the
// eight values of warp w that meet in its (l, l+4) pair, in the tree's own pairing
// ((v_l + v_l+16) + (v_l+8 + v_l+24)) + ((v_l+4 + v_l+20) + (v_l+12 + v_l+28)), then the
// (l, l+2), (l, l+1) levels and the cross-warp levels by shuffles.  12 FP64 warp
// instructions instead of 43 on GB300's narrow FP64 pipe, the same bits; the values sit in
// shared memory with one pad per 32 (fewer bank conflicts on the strided reads).
__device__ __forceinline__ double block_tree256(double v, double* red) {
    __shared__ double tree_v[256 + 8];
    const int t = threadIdx.x;
    tree_v[t + (t >> 5)] = v;
    __syncthreads();
    if (t < 32) {
        const int w = t >> 2, l = t & 3;
        const double* q = tree_v + 33 * w + l;
        const double b0 = (q[0] + q[16]) + (q[8] + q[24]);
        const double b1 = (q[4] + q[20]) + (q[12] + q[28]);
        double c = b0 + b1;
        c = c + __shfl_down_sync(0xffffffffu, c, 2);   // (l, l+2)
        c = c + __shfl_down_sync(0xffffffffu, c, 1);   // (l, l+1): warp w's sum in lane 4w
        c = c + __shfl_down_sync(0xffffffffu, c, 16);  // (w, w+4)
        c = c + __shfl_down_sync(0xffffffffu, c, 8);   // (w, w+2)
        c = c + __shfl_down_sync(0xffffffffu, c, 4);   // (w, w+1)
        if (t == 0) red[8] = c;
    }
    __syncthreads();
    double r = red[8];
    __syncthreads();
    return r;
}

// Final fold of nc chunk partials (blockDim.x == 256); every thread gets the sum.
__device__ __forceinline__ double fold_partials(const double* part, long nc, double* red) {
    const int t = threadIdx.x;
    double acc = (t < nc) ? part[t] : 0.0;
    for (long c = t + 256; c < nc; c += 256) acc = acc + part[c];
    return block_tree256(acc, red);
}

// ------------------------------------------------------------------ bounded waits
// Every device-side wait of the library is bounded twice: by a number of polls and by the
// elapsed time on the GPU's global nanosecond timer (a poll may suspend the thread for a
// system-dependent time, so the count alone does not bound the time).
constexpr long long kSpinLimit = 1LL << 24;
constexpr unsigned long long kWaitNs = 1000000000ull;  // 1 s

__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Sense-free generation barrier for cooperative launches.  A block that waits longer than
// the bounds above sets *err = CFD_ERR_BARRIER and leaves; callers check err.

struct GridBar {
    unsigned int arrive;
    unsigned int gen;
    int err;
    int pad;
};

__device__ __forceinline__ void grid_barrier(GridBar* gb, unsigned nblocks,
                                             long long limit = kSpinLimit) {
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned int* vgen = &gb->gen;
        unsigned int g = *vgen;
        __threadfence();
        unsigned int prev = atomicAdd(&gb->arrive, 1u);
        if (prev == nblocks - 1) {
            atomicExch(&gb->arrive, 0u);
            __threadfence();
            atomicAdd(&gb->gen, 1u);
        } else {
            long long spins = 0;
            const unsigned long long t0 = globaltimer_ns();
            while (*vgen == g) {
                if (++spins > limit ||
                    ((spins & 63) == 0 && globaltimer_ns() - t0 > kWaitNs)) {
                    atomicExch(&gb->err, (int)CFD_ERR_BARRIER);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// Bounded wait on the phase of the given parity of a shared-memory mbarrier (an mbarrier
// completed by bulk copies or by tcgen05.commit): false after `limit` polls or kWaitNs
__device__ __forceinline__ bool mbar_wait_bounded(unsigned ubar, unsigned parity,
                                                  long long limit = kSpinLimit) {
    unsigned done = 0;
    const unsigned long long t0 = globaltimer_ns();
    for (long long k = 0; k < limit && !done; ++k) {
        asm volatile(
            "{ .reg .pred q; mbarrier.try_wait.parity.shared::cta.b64 q, [%1], %2; "
            "selp.u32 %0, 1, 0, q; }"
            : "=r"(done)
            : "r"(ubar), "r"(parity)
            : "memory");
        if (!done && (k & 63) == 63 && globaltimer_ns() - t0 > kWaitNs) break;
    }
    return done != 0;
}

}  // namespace cfd
