// Exact, order-independent sums of doubles (the dec aggregate_sum).
//
// AggregateSum adds dec values with `+=` in whatever order its threads run
// (operators/aggregatesum.cpp:97-102). On the GPU thousands of threads add
// into one group at once, so any floating-point accumulation depends on
// arrival order. Here each value is instead turned into a signed 192-bit
// integer count of units 2^s, and integers add associatively: whatever the
// order, the table ends with the same sum, held in three 64-bit words and
// updated with integer atomics (an add that can carry returns the old word,
// which gives the carry into the next word). The final double is that
// integer times 2^s, rounded once to nearest-even.
//
// The unit: with every finite |x| < 2^(E+1) and at most n values per call,
// s = E + 1 + bits(n) - 190 keeps |sum| < 2^190, inside the signed range.
// A value is held exactly when its ulp is a multiple of 2^s, that is when it
// is at most about 2^(137 - bits(n)) times smaller than the largest value
// (2^109 for 256M rows). When all values are held exactly, the result is the
// correctly rounded exact sum, the value an exact summation (such as Python's
// math.fsum) gives, on every run and launch shape. Smaller values are
// rounded to the unit (ties to even), deterministically. A value near the
// largest occupies the upper two words, so a row costs two atomics. Infinities
// and NaNs are not quantised: the caller tracks them on the side.
//
// Host and device: the host test checks quantisation and rounding against
// exact rational arithmetic.
#ifndef PG_FIXSUM_H
#define PG_FIXSUM_H

#include <stdint.h>
#include <string.h>

#if defined(__CUDACC__)
#define PG_FX_HD __host__ __device__ __forceinline__
#else
#define PG_FX_HD static inline
#endif

#define PG_FX_EXP_SPECIAL 0x7FF      // exponent field of infinities and NaNs

// A signed 192-bit count, two's complement, w0 least significant.
struct pg_fx3 {
	uint64_t w0, w1, w2;
};

PG_FX_HD int pg_fx_clz64(uint64_t x)
{
#if defined(__CUDA_ARCH__)
	return __clzll((long long) x);
#else
	return x ? __builtin_clzll(x) : 64;
#endif
}

// Exponent field (biased) of the double with bit pattern b.
PG_FX_HD int pg_fx_field(uint64_t b)
{
	return (int) ((b >> 52) & 0x7FF);
}

// Unit exponent s for values whose exponent field is at most `field` (the
// largest finite field seen, or a bound on it), n values at most.
PG_FX_HD int pg_fx_unit(int field, uint64_t n)
{
	if (field < 1) field = 1;                               // zeros and subnormals only
	const int nbits = 64 - pg_fx_clz64(n | 1);
	return field - 1212 + nbits;                            // (field - 1023 + 1) + bits(n) - 190
}

PG_FX_HD void pg_fx_neg(pg_fx3& a)
{
	a.w0 = ~a.w0 + 1;
	uint64_t c = a.w0 == 0;
	a.w1 = ~a.w1 + c;
	c = c && a.w1 == 0;
	a.w2 = ~a.w2 + c;
}

// The finite double with bit pattern b (field <= the bound s was made from)
// as a signed count of units 2^s, rounded to nearest, ties to even.
PG_FX_HD pg_fx3 pg_fx_quant(uint64_t b, int s)
{
	const int e = pg_fx_field(b);
	uint64_t mant = b & 0xFFFFFFFFFFFFFull;
	if (e) mant |= 1ull << 52;
	const int sh = (e ? e : 1) - 1075 - s;                  // |x| = mant * 2^(s + sh), sh <= 136
	pg_fx3 r = {0, 0, 0};
	if (sh >= 0) {
		const int bit = sh & 63;
		const uint64_t lo = mant << bit, hi = bit ? mant >> (64 - bit) : 0;
		if (sh < 64) { r.w0 = lo; r.w1 = hi; }
		else if (sh < 128) { r.w1 = lo; r.w2 = hi; }
		else r.w2 = lo;                                     // mant << (sh - 128) < 2^62
	} else {
		const int rs = -sh;
		if (rs <= 54) {                                     // below: under a quarter unit
			uint64_t q = mant >> rs;
			const uint64_t rem = mant & ((1ull << rs) - 1), half = 1ull << (rs - 1);
			if (rem > half || (rem == half && (q & 1))) ++q;
			r.w0 = q;
		}
	}
	if (b >> 63) pg_fx_neg(r);
	return r;
}

// a += b, modulo 2^192.
PG_FX_HD void pg_fx_add(pg_fx3& a, const pg_fx3& b)
{
	const uint64_t l = a.w0 + b.w0;
	uint64_t c = l < a.w0;
	a.w0 = l;
	const uint64_t m = a.w1 + b.w1;
	const uint64_t c1 = m < a.w1;
	a.w1 = m + c;
	c = c1 + (a.w1 < c);
	a.w2 += b.w2 + c;
}

// Bit i of a (0 <= i < 192).
PG_FX_HD uint64_t pg_fx_bit(const pg_fx3& a, int i)
{
	const uint64_t w = i < 64 ? a.w0 : i < 128 ? a.w1 : a.w2;
	return (w >> (i & 63)) & 1;
}

// 64 bits of a from bit i up (i >= 0; bits past 191 read as 0).
PG_FX_HD uint64_t pg_fx_window(const pg_fx3& a, int i)
{
	const int k = i >> 6, bit = i & 63;
	const uint64_t w = k == 0 ? a.w0 : k == 1 ? a.w1 : k == 2 ? a.w2 : 0;
	const uint64_t n = k == 0 ? a.w1 : k == 1 ? a.w2 : 0;
	return bit ? (w >> bit) | (n << (64 - bit)) : w;
}

// Whether any of bits 0 .. i-1 of a is set.
PG_FX_HD bool pg_fx_any_below(const pg_fx3& a, int i)
{
	if (i <= 0) return false;
	const uint64_t m0 = i >= 64 ? ~0ull : (1ull << i) - 1;
	const uint64_t m1 = i >= 128 ? ~0ull : i > 64 ? (1ull << (i - 64)) - 1 : 0;
	const uint64_t m2 = i > 128 ? (1ull << (i - 128)) - 1 : 0;
	return (a.w0 & m0) || (a.w1 & m1) || (a.w2 & m2);
}

// The signed count a of units 2^s as a double, rounded to nearest, ties to
// even (subnormal and infinite results included). A zero count gives +0.0,
// as the reference's sum from 0.0 does.
PG_FX_HD double pg_fx_double(pg_fx3 a, int s)
{
	const uint64_t sign = a.w2 & (1ull << 63);
	if (sign) pg_fx_neg(a);
	uint64_t bits = 0;
	if (a.w0 | a.w1 | a.w2) {
		const int p = a.w2 ? 192 - pg_fx_clz64(a.w2) : a.w1 ? 128 - pg_fx_clz64(a.w1) : 64 - pg_fx_clz64(a.w0);
		int t = s + p - 53;                                  // exponent of the result's last bit
		if (t < -1074) t = -1074;
		const int sh = t - s;                                // bits dropped
		uint64_t m;
		if (sh <= 0) m = a.w0 << (-sh);                      // p <= 53: exact
		else {
			m = pg_fx_window(a, sh) & ((1ull << 54) - 1);
			if (pg_fx_bit(a, sh - 1) && (pg_fx_any_below(a, sh - 1) || (m & 1))) ++m;
			if (m == (1ull << 53)) { m >>= 1; ++t; }
		}
		if (m < (1ull << 52)) bits = m;                      // subnormal (t = -1074)
		else {
			const int biased = t + 52 + 1023;
			bits = biased >= 2047 ? 0x7FF0000000000000ull
			                      : ((uint64_t) biased << 52) | (m & 0xFFFFFFFFFFFFFull);
		}
	}
	bits |= sign;
	double x;
#if defined(__CUDA_ARCH__)
	x = __longlong_as_double((long long) bits);
#else
	memcpy(&x, &bits, 8);
#endif
	return x;
}

// Side flags of a dec sum, per group, for values that are not quantised.
#define PG_FX_POS_INF 1u
#define PG_FX_NEG_INF 2u
#define PG_FX_NAN 4u

PG_FX_HD uint32_t pg_fx_special(uint64_t b)
{
	if (b & 0xFFFFFFFFFFFFFull) return PG_FX_NAN;
	return (b >> 63) ? PG_FX_NEG_INF : PG_FX_POS_INF;
}

// IEEE result of a sum that met the special values in `flags`.
PG_FX_HD uint64_t pg_fx_special_bits(uint32_t flags)
{
	if ((flags & PG_FX_NAN) || (flags & (PG_FX_POS_INF | PG_FX_NEG_INF)) == (PG_FX_POS_INF | PG_FX_NEG_INF))
		return 0x7FF8000000000000ull;
	return (flags & PG_FX_NEG_INF) ? 0xFFF0000000000000ull : 0x7FF0000000000000ull;
}

#endif
