// Correctly rounded FP64 multiply and add computed on the integer pipes.
//
// The GB300's FP64 pipe issues two thread-operations per SM per cycle, while
// its integer pipes (ALU and the integer multiply-add path) together take about
// one warp instruction per scheduler per cycle.  An FP64 kernel that keeps the
// FP64 pipe busy leaves the integer issue slots almost idle; an operation moved
// there runs concurrently with the hardware ones.  The results are bit for bit
// the IEEE 754 binary64 round-to-nearest-even results, so moving an operation
// changes no result.
//
// Method: the classic sign / exponent / significand decomposition with guard
// and sticky bits (IEEE 754-2019 section 4.3.1 defines the rounding; the
// algorithms are those of Muller et al., "Handbook of Floating-Point
// Arithmetic", 2nd ed., 2018, ch. 7, "Algorithms for the five basic
// operations": the product and the sum, with a sticky bit folded into the
// least significant bit of the aligned operand).  Only the common case is
// handled here: finite normal operands whose result is normal (and, for the
// sum, not an exact zero), and for the product also a zero times a finite
// number.  Every other case -- other zeros, subnormals, infinities, NaN,
// results that underflow or overflow -- calls the hardware instruction, so the
// functions are total.  The probe kernels in probe.cu test them bit for
// bit against the hardware instructions and time them.
//
// The functions compile for the host as well (the fallback is then the host's
// own IEEE operation), so that the same code is tested against numpy on the CPU.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

namespace fvgb {
namespace soft {

// The bit moves go through inline PTX on the device: the compiler recognises a bit cast
// followed by a sign mask or flip as fabs or negation and issues it as an FP64 instruction,
// on the pipe these functions exist to relieve.
__host__ __device__ __forceinline__ uint64_t bits_of(double x) {
#if defined(__CUDA_ARCH__)
    uint64_t u;
    asm("mov.b64 %0, %1;" : "=l"(u) : "d"(x));
    return u;
#else
    uint64_t u;
    memcpy(&u, &x, sizeof u);
    return u;
#endif
}
__host__ __device__ __forceinline__ double double_of(uint64_t u) {
#if defined(__CUDA_ARCH__)
    double x;
    asm("mov.b64 %0, %1;" : "=d"(x) : "l"(u));
    return x;
#else
    double x;
    memcpy(&x, &u, sizeof x);
    return x;
#endif
}

// The rare cases call these out-of-line functions.  A call is a real branch: inlined,
// the fallback instruction would be if-converted into a predicated FP64 instruction
// that issues on every call and holds the FP64 pipe that the integer path exists to
// relieve.
#if defined(__CUDA_ARCH__)
static __device__ __noinline__ double mul_rare(double a, double b) { return __dmul_rn(a, b); }
static __device__ __noinline__ double add_rare(double a, double b) { return __dadd_rn(a, b); }
#else
static inline double mul_rare(double a, double b) {
    volatile double r = a * b;
    return r;
}
static inline double add_rare(double a, double b) {
    volatile double r = a + b;
    return r;
}
#endif

__host__ __device__ __forceinline__ int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}

constexpr uint64_t kSign = 0x8000000000000000ull;
constexpr uint64_t kFrac = 0x000fffffffffffffull;
constexpr uint64_t kHidden = 0x0010000000000000ull;

// a * b, round to nearest even
__host__ __device__ __forceinline__ double dmul(double a, double b) {
    const uint64_t ua = bits_of(a), ub = bits_of(b);
    const uint32_t ha = (uint32_t)(ua >> 32), hb = (uint32_t)(ub >> 32);
    const int ea = (int)((ha >> 20) & 0x7ffu), eb = (int)((hb >> 20) & 0x7ffu);
    const int e = ea + eb - 1023;  // biased exponent when the significands' product lies in [1, 2)
    // normal operands and a normal result even after a normalising shift and a rounding carry
    if (!((unsigned)(ea - 1) < 2046u && (unsigned)(eb - 1) < 2046u && (unsigned)(e - 1) < 2044u)) {
        // a zero times a finite number is a zero with the sign of the product: common where
        // a field is uniform or an adjoint is zero, and no reason to leave the integer pipe
        const bool za = (ua << 1) == 0ull, zb = (ub << 1) == 0ull;
        if ((za && eb != 0x7ff) || (zb && ea != 0x7ff)) return double_of((ua ^ ub) & kSign);
        return mul_rare(a, b);
    }
    // significands ma 2^32 + la and mb 2^32 + lb (53 bits each, hidden bit set)
    const uint32_t la = (uint32_t)ua, lb = (uint32_t)ub;
    const uint32_t ma = (ha & 0xfffffu) | 0x100000u, mb = (hb & 0xfffffu) | 0x100000u;
    // the exact 106-bit product P = hi 2^64 + (mid mod 2^32) 2^32 + (ll mod 2^32), 2^104 <= P < 2^106
    const uint64_t ll = (uint64_t)la * lb;
    const uint64_t mid = (uint64_t)la * mb + (uint64_t)ma * lb + (ll >> 32);
    const uint64_t hi = (uint64_t)ma * mb + (mid >> 32);
    const uint32_t midlo = (uint32_t)mid;
    const uint64_t t = (hi << 13) | (midlo >> 19);            // P >> 51: 54 bits, or 55 when P >= 2^105
    const uint32_t sticky = (midlo & 0x7ffffu) | (uint32_t)ll;  // P mod 2^51
    const int n = (int)(t >> 54);                              // 1 when P >= 2^105
    const uint64_t m = t >> (1 + n);                           // the 53-bit significand, truncated
    const uint32_t guard = (uint32_t)(t >> n) & 1u;
    const bool rest = (sticky | ((uint32_t)t & (uint32_t)n)) != 0u;  // everything below the guard bit
    const uint64_t inc = guard & ((uint32_t)rest | ((uint32_t)m & 1u));
    // the hidden bit of m adds one to the exponent field; a rounding carry to 2^53 adds one more
    const uint64_t bits = ((uint64_t)(e + n - 1) << 52) + m + inc;
    return double_of(bits | ((ua ^ ub) & kSign));
}

// a + b, round to nearest even
__host__ __device__ __forceinline__ double dadd(double a, double b) {
    uint64_t ua = bits_of(a), ub = bits_of(b);
    uint64_t aa = ua & ~kSign, ab = ub & ~kSign;
    if (ab > aa) {  // |a| >= |b| from here on
        const uint64_t t = ua;
        ua = ub;
        ub = t;
        const uint64_t s = aa;
        aa = ab;
        ab = s;
    }
    const int ea = (int)(aa >> 52), eb = (int)(ab >> 52);
    if (!((unsigned)(ea - 1) < 2046u && (unsigned)(eb - 1) < 2046u)) return add_rare(a, b);
    // significands with ten guard bits: the hidden bit sits at bit 62
    const uint64_t ma = ((aa & kFrac) | kHidden) << 10;
    const uint64_t mb = ((ab & kFrac) | kHidden) << 10;
    const int d = (ea - eb < 63) ? ea - eb : 63;
    // b aligned to a, the bits shifted out folded into a sticky least significant bit
    const uint64_t mbs = (mb >> d) | (uint64_t)((mb & ((1ull << d) - 1ull)) != 0ull);
    const bool sub = ((ua ^ ub) & kSign) != 0ull;
    uint64_t r = sub ? ma - mbs : ma + mbs;
    if (r == 0ull) return add_rare(a, b);  // exact cancellation: +0
    // normalise to the hidden bit at bit 62: one right shift (keeping the sticky bit) after a
    // carry, or a left shift after cancellation (exact, or by one place when bits were lost)
    const int lz = clz64(r);
    int e = ea;
    if (lz == 0) {
        r = (r >> 1) | (r & 1ull);
        e += 1;
    } else {
        r <<= (lz - 1);
        e -= (lz - 1);
    }
    if (!((unsigned)(e - 1) < 2045u)) return add_rare(a, b);  // underflow, or overflow after rounding
    const uint64_t m = r >> 10;
    const uint32_t low = (uint32_t)r & 0x3ffu;  // guard bit 9, then the rest
    const uint64_t inc = (low > 0x200u || (low == 0x200u && (m & 1ull))) ? 1ull : 0ull;
    const uint64_t bits = ((uint64_t)(e - 1) << 52) + m + inc;
    return double_of(bits | (ua & kSign));
}

__host__ __device__ __forceinline__ double dsub(double a, double b) { return dadd(a, double_of(bits_of(b) ^ kSign)); }

}  // namespace soft
}  // namespace fvgb
