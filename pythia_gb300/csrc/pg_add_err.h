// Exact rounding error of a double addition, in integer arithmetic.
//
// pg_add_err(a, b) returns e = (a + b) - RN(a + b) exactly, where RN is IEEE
// round-to-nearest-even: the value Knuth's TwoSum (or Dekker's Fast2Sum)
// computes with six (three) FP64 additions. It is computed here from the bit
// patterns: both significands are aligned at the smaller operand's exponent
// in a 128-bit integer (an exponent gap above 54 bits means the smaller
// operand is below a quarter ulp of the larger one, so it is the error
// itself), the exact sum is rounded to 53 significant bits (ties to even),
// and the remainder, which is exactly representable, is rebuilt as a double
// (normal or subnormal). Infinite or NaN operands give 0.
//
// On GPUs whose FP64 pipe is narrow, a compensated aggregation spends most of
// its instruction time in those FP64 additions; this version uses only
// 64/128-bit integer operations. It compiles for host and device so that the
// host test checks it bit for bit against TwoSum.
#ifndef PG_ADD_ERR_H
#define PG_ADD_ERR_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define PG_AE_HD __host__ __device__ __forceinline__
#else
#define PG_AE_HD static inline
#endif

PG_AE_HD int pg_ae_clz64(uint64_t x)
{
#if defined(__CUDA_ARCH__)
	return __clzll((long long) x);
#else
	return x ? __builtin_clzll(x) : 64;
#endif
}

PG_AE_HD uint64_t pg_ae_bits(double x)
{
#if defined(__CUDA_ARCH__)
	return (uint64_t) __double_as_longlong(x);
#else
	uint64_t u;
	memcpy(&u, &x, 8);
	return u;
#endif
}

PG_AE_HD double pg_ae_double(uint64_t u)
{
#if defined(__CUDA_ARCH__)
	return __longlong_as_double((long long) u);
#else
	double x;
	memcpy(&x, &u, 8);
	return x;
#endif
}

// Bit pattern of e = (a + b) - RN(a + b) for bit patterns ua, ub.
PG_AE_HD uint64_t pg_add_err_bits(uint64_t ua, uint64_t ub)
{
	const uint64_t ABS = 0x7FFFFFFFFFFFFFFFull, FRAC = 0x000FFFFFFFFFFFFFull;
	uint64_t xa = ua & ABS, xb = ub & ABS;
	if (xa < xb) { uint64_t t = ua; ua = ub; ub = t; t = xa; xa = xb; xb = t; }   // |a| >= |b|
	if (xb == 0) return 0;                                  // b = ±0: exact
	int ea = (int) (xa >> 52), eb = (int) (xb >> 52);
	if (ea == 0x7FF) return 0;                              // inf / nan
	uint64_t ma = xa & FRAC, mb = xb & FRAC;
	if (ea) ma |= 1ull << 52; else ea = 1;
	if (eb) mb |= 1ull << 52; else eb = 1;
	const int d = ea - eb;
	if (d > 54) return ub;                                  // |b| < ulp(a) / 4: RN(a + b) = a
	// Exact sum at exponent eb: a's significand shifted left by d (<= 107 bits).
	const unsigned __int128 A = (unsigned __int128) ma << d, B = mb;
	const bool neg = (ua >> 63) != 0;                       // the sum takes a's sign
	const unsigned __int128 M = ((ua ^ ub) >> 63) ? A - B : A + B;
	if (M == 0) return 0;
	const uint64_t mh = (uint64_t) (M >> 64), ml = (uint64_t) M;
	const int nb = mh ? 128 - pg_ae_clz64(mh) : 64 - pg_ae_clz64(ml);
	if (nb <= 53) return 0;                                 // the sum fits 53 bits
	const int sh = nb - 53;                                 // 1..55
	const unsigned __int128 one = 1;
	const unsigned __int128 r = M & ((one << sh) - 1);
	const unsigned __int128 half = one << (sh - 1);
	const bool qodd = (uint64_t) (M >> sh) & 1;
	// Rounded result exponent overflows: the sum is infinite, no finite error.
	if (eb + sh + 52 >= 0x7FF + 52) return 0;
	// Error magnitude in units of 2^(eb - 1075): r (rounded down) or
	// 2^sh - r (rounded up); the error's sign is a's when rounding down.
	bool eneg;
	unsigned __int128 mag;
	if (r > half || (r == half && qodd)) { mag = (one << sh) - r; eneg = !neg; }
	else { mag = r; eneg = neg; }
	if (mag == 0) return 0;
	// mag < 2^55 and has at most 53 significant bits (the error is a double).
	const uint64_t m = (uint64_t) mag;
	const int mbits = 64 - pg_ae_clz64(m);
	const int be = eb + mbits - 53;                         // biased exponent if normal
	uint64_t bits;
	if (be >= 1) {
		const uint64_t sig = mbits <= 53 ? m << (53 - mbits) : m >> (mbits - 53);
		bits = ((uint64_t) be << 52) | (sig & FRAC);
	} else {
		bits = m << (eb - 1);                               // subnormal: m * 2^(eb - 1075)
	}
	return bits | ((uint64_t) eneg << 63);
}

PG_AE_HD double pg_add_err(double a, double b)
{
	return pg_ae_double(pg_add_err_bits(pg_ae_bits(a), pg_ae_bits(b)));
}

#endif
