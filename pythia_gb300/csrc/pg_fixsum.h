// Exact, order-independent sums of doubles (the dec aggregate_sum).
//
// AggregateSum adds dec values with `+=` in whatever order its threads run
// (operators/aggregatesum.cpp:97-102). On the GPU thousands of threads add
// into one group at once, so any floating-point accumulation depends on
// arrival order. Here each value is instead turned into a signed integer
// count of units 2^s, and integers add associatively: whatever the order, the
// table ends with the same sum, held in seven 64-bit words and updated with
// integer atomics. The final double is that integer times 2^s, rounded once
// to nearest-even.
//
// The unit: with every finite |x| < 2^(E+1), s = E + 1 - 128 - PG_FX_TOP, so
// a value's count is below 2^(128 + PG_FX_TOP): it fits in three words, and
// a value within 2^(PG_FX_TOP - 53) of the largest lies wholly in the third.
// A value is held exactly when its ulp is a multiple of 2^s, that is when it
// is at most 2^(PG_FX_TOP + 75) times smaller than the largest. When all
// values are held exactly, the result is the correctly rounded exact sum, the
// value an exact summation (such as Python's math.fsum) gives, on every run
// and launch shape. Smaller values are rounded to the unit (ties to even),
// deterministically. Infinities and NaNs are not quantised: the caller tracks
// them on the side.
//
// A group's table slot: t2 (signed) and t3 hold the count's bits from 128 up,
// the sum being t3 2^192 + t2 2^128 + ...; an add into t2 returns the old
// word, whose signed overflow adds +-1 into t3. The low 128 bits go, as
// 28-bit chunks, into five lazy words l0..l4 (chunk k into lk, weight 2^28k)
// with adds that return nothing: a word that takes fewer than 2^36 chunks
// cannot overflow, and a group takes at most one chunk per word per row (a
// device-resident column of 8-byte values has fewer than 2^36 rows). So a
// value near the column's largest, whose low bits are zero, costs one
// returning atomic, t2 overflows only about once per 2^(64 - PG_FX_TOP) such
// values, and values far below the largest add fire-and-forget chunks.
// Tables in shared memory, where returning adds are cheap, use a compact
// four-word chained form instead (pg_fx_chain_add).
//
// Host and device: the host test checks quantisation, both table forms' adds
// and the rounding against exact rational arithmetic.
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
#define PG_FX_TOP 60                 // bits of the third word a value of the bound's binade fills

// Words of a group's table, word k at t[k * stride] (the GPU's dense tables
// keep each word in an array of its own, so that t2, which every row adds
// into, takes 8 bytes a group of L2).
#define PG_FX_T2 0                   // count bits 128..191, signed
#define PG_FX_T3 1                   // t2's signed overflows and count bits from 192
#define PG_FX_L0 2                   // lazy words l0..l4: sums of 28-bit chunks of bits 0..127
#define PG_FX_LAZY 5
#define PG_FX_CHUNK 28
#define PG_FX_WORDS 7

// One value's count: signed 192-bit, two's complement, w0 least significant.
struct pg_fx3 {
	uint64_t w0, w1, w2;
};

// A signed 256-bit count, two's complement (sums of values).
struct pg_fx4 {
	uint64_t w0, w1, w2, w3;
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
// largest finite field seen, or a bound on it).
PG_FX_HD int pg_fx_unit(int field)
{
	if (field < 1) field = 1;                               // zeros and subnormals only
	return field - 1150 - PG_FX_TOP;                        // (field - 1023 + 1) - 128 - PG_FX_TOP
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
	const int sh = (e ? e : 1) - 1075 - s;                  // |x| = mant * 2^(s + sh), sh <= 75 + PG_FX_TOP
	pg_fx3 r = {0, 0, 0};
	if (sh >= 0) {
		const int bit = sh & 63;
		const uint64_t lo = mant << bit, hi = bit ? mant >> (64 - bit) : 0;
		if (sh < 64) { r.w0 = lo; r.w1 = hi; }
		else if (sh < 128) { r.w1 = lo; r.w2 = hi; }
		else r.w2 = lo;                                     // mant << (sh - 128) < 2^PG_FX_TOP
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

// The 256-bit count of a value's 192-bit one (sign-extended).
PG_FX_HD pg_fx4 pg_fx_widen(const pg_fx3& a)
{
	return pg_fx4{a.w0, a.w1, a.w2, (uint64_t) ((int64_t) a.w2 >> 63)};
}

// Adds y and the carry c (0 or 1) to x; returns the carry out.
PG_FX_HD uint64_t pg_fx_adc(uint64_t& x, uint64_t y, uint64_t c)
{
	const uint64_t s1 = x + y;
	const uint64_t c1 = s1 < y;
	x = s1 + c;
	return c1 + (x < c);
}

// a += b, modulo 2^256.
PG_FX_HD void pg_fx_add4(pg_fx4& a, const pg_fx4& b)
{
	uint64_t c = pg_fx_adc(a.w0, b.w0, 0);
	c = pg_fx_adc(a.w1, b.w1, c);
	c = pg_fx_adc(a.w2, b.w2, c);
	a.w3 += b.w3 + c;
}

// Chunk k (PG_FX_CHUNK bits from bit 28k) of the 128-bit (hi, lo).
PG_FX_HD uint64_t pg_fx_chunk(uint64_t lo, uint64_t hi, int k)
{
	const int b = PG_FX_CHUNK * k;
	const uint64_t w = b == 0 ? lo : b < 64 ? (lo >> b) | (hi << (64 - b)) : hi >> (b - 64);
	return w & ((1ull << PG_FX_CHUNK) - 1);
}

// The count held by table words t[k * stride] (k < PG_FX_WORDS).
PG_FX_HD pg_fx4 pg_fx_from_table(const uint64_t* t, uint64_t stride)
{
	const uint64_t t2 = t[PG_FX_T2 * stride];
	pg_fx4 a = {0, 0, t2, t[PG_FX_T3 * stride] - (t2 >> 63)};
	for (int k = 0; k < PG_FX_LAZY; ++k) {
		const uint64_t l = t[(PG_FX_L0 + k) * stride];
		const int b = PG_FX_CHUNK * k;                     // l 2^b, l < 2^64
		pg_fx4 c = {0, 0, 0, 0};
		if (b == 0) c.w0 = l;
		else if (b < 64) { c.w0 = l << b; c.w1 = l >> (64 - b); }
		else if (b == 64) c.w1 = l;
		else { c.w1 = l << (b - 64); c.w2 = l >> (128 - b); }
		pg_fx_add4(a, c);
	}
	return a;
}

// The upper part of count a, a3 2^192 + a2 2^128, as r 2^128 + q 2^192 with
// r a signed 64-bit word (what goes into t2 and t3).
PG_FX_HD void pg_fx_split_top(uint64_t a2, uint64_t a3, int64_t& r, uint64_t& q)
{
	q = a3 + (a2 >> 63);
	r = (int64_t) a2;
}

// The +-1 that adding r to a signed word whose old value was `old` carries
// into the next word (its signed overflow).
PG_FX_HD uint64_t pg_fx_overflow(uint64_t old, int64_t r)
{
	const int64_t o = (int64_t) old, w = (int64_t) (old + (uint64_t) r);
	return r > 0 ? (uint64_t) (w < o) : (w > o ? ~0ull : 0);
}

// Adds count a into table words t[k * stride] (k < PG_FX_WORDS) one add at a
// time, as the atomics do: ADD(p, v) adds v at p and returns the old word.
// Returns whether the add into t2 returned 0, or none was made (the group's
// first row marks it present).
template <class ADD>
PG_FX_HD bool pg_fx_table_add(uint64_t* t, uint64_t stride, const pg_fx4& a, ADD add)
{
	int64_t r;
	uint64_t q;
	pg_fx_split_top(a.w2, a.w3, r, q);
	bool mark = true;
	if (r) {
		const uint64_t old = add(t + PG_FX_T2 * stride, (uint64_t) r);
		q += pg_fx_overflow(old, r);
		mark = old == 0;
	}
	if (q) add(t + PG_FX_T3 * stride, q);
	for (int k = 0; k < PG_FX_LAZY; ++k) {
		const uint64_t c = pg_fx_chunk(a.w0, a.w1, k);
		if (c) add(t + (PG_FX_L0 + k) * stride, c);
	}
	return mark;
}

// A compact four-word form for tables in shared memory, where returning
// adds are cheap: t[0], t[1] unsigned, t[2] signed, t[3] its overflows, the
// sum being t3 2^192 + t2 2^128 + t1 2^64 + t0. Each add returns the old word,
// whose overflow is the carry into the next word.
template <class ADD>
PG_FX_HD void pg_fx_chain_add(uint64_t* t, uint64_t stride, const pg_fx4& a, ADD add)
{
	uint64_t c = 0;
	if (a.w0) {
		const uint64_t old = add(t, a.w0);
		c = old + a.w0 < old;
	}
	const uint64_t x1 = a.w1 + c;
	c = x1 < c;
	if (x1) {
		const uint64_t old = add(t + stride, x1);
		c += old + x1 < old;
	}
	const uint64_t l = a.w2 + c;                           // the rest: (a3 + carry) 2^192 + l 2^128
	uint64_t q = a.w3 + (l < c) + (l >> 63);
	const int64_t r = (int64_t) l;
	if (r) q += pg_fx_overflow(add(t + 2 * stride, (uint64_t) r), r);
	if (q) add(t + 3 * stride, q);
}

// The count held by a four-word chained table t[k * stride].
PG_FX_HD pg_fx4 pg_fx_from_chain(const uint64_t* t, uint64_t stride)
{
	const uint64_t t2 = t[2 * stride];
	return pg_fx4{t[0], t[stride], t2, t[3 * stride] - (t2 >> 63)};
}

PG_FX_HD void pg_fx_neg4(pg_fx4& a)
{
	a.w0 = ~a.w0; a.w1 = ~a.w1; a.w2 = ~a.w2; a.w3 = ~a.w3;
	uint64_t c = pg_fx_adc(a.w0, 1, 0);
	c = pg_fx_adc(a.w1, 0, c);
	c = pg_fx_adc(a.w2, 0, c);
	a.w3 += c;
}

PG_FX_HD uint64_t pg_fx_word(const pg_fx4& a, int k)
{
	return k == 0 ? a.w0 : k == 1 ? a.w1 : k == 2 ? a.w2 : k == 3 ? a.w3 : 0;
}

// Bit i of a (0 <= i < 256).
PG_FX_HD uint64_t pg_fx_bit(const pg_fx4& a, int i)
{
	return (pg_fx_word(a, i >> 6) >> (i & 63)) & 1;
}

// 64 bits of a from bit i up (i >= 0; bits past 255 read as 0).
PG_FX_HD uint64_t pg_fx_window(const pg_fx4& a, int i)
{
	const int k = i >> 6, bit = i & 63;
	const uint64_t w = pg_fx_word(a, k), n = pg_fx_word(a, k + 1);
	return bit ? (w >> bit) | (n << (64 - bit)) : w;
}

// Whether any of bits 0 .. i-1 of a is set.
PG_FX_HD bool pg_fx_any_below(const pg_fx4& a, int i)
{
	for (int k = 0; k < 4 && i > 0; ++k, i -= 64) {
		const uint64_t m = i >= 64 ? ~0ull : (1ull << i) - 1;
		if (pg_fx_word(a, k) & m) return true;
	}
	return false;
}

// The signed count a of units 2^s as a double, rounded to nearest, ties to
// even (subnormal and infinite results included). A zero count gives +0.0,
// as the reference's sum from 0.0 does.
PG_FX_HD double pg_fx_double4(pg_fx4 a, int s)
{
	const uint64_t sign = a.w3 & (1ull << 63);
	if (sign) pg_fx_neg4(a);
	uint64_t bits = 0;
	if (a.w0 | a.w1 | a.w2 | a.w3) {
		const int p = a.w3 ? 256 - pg_fx_clz64(a.w3) : a.w2 ? 192 - pg_fx_clz64(a.w2)
		            : a.w1 ? 128 - pg_fx_clz64(a.w1) : 64 - pg_fx_clz64(a.w0);
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

// The sum held by table words t[k * stride] as a double.
PG_FX_HD double pg_fx_table_double(const uint64_t* t, uint64_t stride, int s)
{
	return pg_fx_double4(pg_fx_from_table(t, stride), s);
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
