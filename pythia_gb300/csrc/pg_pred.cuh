// Column predicates of Filter (operators/filter.cpp:37-85): a column compared
// with a constant of the column's own type through Comparator
// (comparator.cpp:43-433) and its raw functions (rawcompfns.cpp): int, long
// and date as signed integers, dec as double (IEEE comparisons, so NaN is
// unequal to everything), char as strncmp over the column width. A set of
// predicates is their conjunction (a Filter over a Filter).
#ifndef PG_PRED_CUH
#define PG_PRED_CUH

#include "pg_internal.cuh"

// Predicates for a kernel parameter; char constants live in device memory
// (PG_PRED_MAX x 128 bytes at `chars`).
struct PgPredSet {
	int n;
	uint32_t type[PG_PRED_MAX], op[PG_PRED_MAX], off[PG_PRED_MAX], bytes[PG_PRED_MAX];
	uint64_t v[PG_PRED_MAX];
	const uint8_t* chars;
};

// Predicates on int/long/dec columns inside a 16-byte tuple held in
// registers (the fused probe prologue).
struct PgPred16 {
	int n;
	uint8_t word[PG_PRED_MAX], type[PG_PRED_MAX], op[PG_PRED_MAX];
	uint64_t v[PG_PRED_MAX];
};

template <typename T>
__device__ __forceinline__ bool pg_cmp(uint32_t op, T a, T b)
{
	switch (op) {
	case PG_CMP_EQ: return a == b;
	case PG_CMP_NE: return a != b;
	case PG_CMP_LT: return a < b;
	case PG_CMP_LE: return a <= b;
	case PG_CMP_GT: return a > b;
	default: return a >= b;
	}
}

// One int/long/dec comparison on the column's bits (lo word, hi word).
__device__ __forceinline__ bool pg_pred_num(uint32_t type, uint32_t op, uint32_t lo, uint32_t hi, uint64_t v)
{
	if (type == PG_PRED_INT) return pg_cmp<int32_t>(op, (int32_t) lo, (int32_t) (uint32_t) v);
	const uint64_t u = ((uint64_t) hi << 32) | lo;
	if (type == PG_PRED_LONG) return pg_cmp<int64_t>(op, (int64_t) u, (int64_t) v);
	return pg_cmp<double>(op, __longlong_as_double((long long) u), __longlong_as_double((long long) v));
}

// The tuple at t (4-byte aligned) satisfies every predicate.
__device__ __forceinline__ bool pg_pred_eval(const PgPredSet& P, const char* __restrict__ t)
{
	#pragma unroll
	for (int i = 0; i < PG_PRED_MAX; ++i) {
		if (i >= P.n) break;
		const char* c = t + P.off[i];
		bool ok;
		if (P.type[i] == PG_PRED_CHAR) {
			// strncmp: the first differing byte decides (as unsigned char);
			// a NUL in both ends the comparison.
			const uint8_t* k = P.chars + i * 128;
			int d = 0;
			for (uint32_t b = 0; b < P.bytes[i]; ++b) {
				const uint8_t x = (uint8_t) c[b], y = k[b];
				if (x != y) { d = x < y ? -1 : 1; break; }
				if (x == 0) break;
			}
			ok = pg_cmp<int>(P.op[i], d, 0);
		} else {
			const uint32_t lo = *reinterpret_cast<const uint32_t*>(c);
			const uint32_t hi = P.type[i] == PG_PRED_INT ? 0 : *reinterpret_cast<const uint32_t*>(c + 4);
			ok = pg_pred_num(P.type[i], P.op[i], lo, hi, P.v[i]);
		}
		if (!ok) return false;
	}
	return true;
}

__device__ __forceinline__ uint32_t pg_word4(const uint4& t, uint32_t w)
{
	return w == 0 ? t.x : w == 1 ? t.y : w == 2 ? t.z : t.w;
}

__device__ __forceinline__ bool pg_pred16(const PgPred16& P, const uint4& t)
{
	bool ok = true;
	#pragma unroll
	for (int i = 0; i < PG_PRED_MAX; ++i)
		if (i < P.n)
			ok = ok && pg_pred_num(P.type[i], P.op[i], pg_word4(t, P.word[i]),
					P.type[i] == PG_PRED_INT ? 0u : pg_word4(t, P.word[i] + 1u), P.v[i]);
	return ok;
}

// Host side: checks `preds` against tuples of `width` bytes; fills the
// kernel form (chars: caller's device copy of the char constants, or null
// when there are none). Returns a PG_ERR_* code.
int pg_pred_prepare(pg_ctx* ctx, const pg_pred* preds, int npred, uint32_t width, PgPredSet* out,
		bool* has_char);
// The register form, when every predicate is an int/long/dec column inside a
// 16-byte tuple; false otherwise.
bool pg_pred_as16(const pg_pred* preds, int npred, PgPred16* out);

#endif
