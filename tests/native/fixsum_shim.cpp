// Host entry points over pythia_gb300/csrc/pg_fixsum.h for the Python test:
// quantisation of doubles to counts of units 2^s, the table adds of the GPU
// kernels (run here one at a time, with plain adds in place of atomics) and
// the rounding of a count back to a double, checked there against exact
// fractions.
#include "pg_fixsum.h"

static uint64_t plain_add(uint64_t* p, uint64_t v)
{
	const uint64_t old = *p;
	*p = old + v;
	return old;
}

extern "C" int fx_unit(int field) { return pg_fx_unit(field); }

extern "C" int fx_words() { return PG_FX_WORDS; }

extern "C" int fx_field(double x)
{
	uint64_t b;
	memcpy(&b, &x, 8);
	return pg_fx_field(b);
}

// Sums xs[0..n) (all finite, fields <= the bound s was made from) into table
// words t[0..PG_FX_WORDS) as the GPU kernels do, in the given order; returns
// the double.
extern "C" double fx_sum(const double* xs, uint64_t n, int s, uint64_t* t)
{
	for (int k = 0; k < PG_FX_WORDS; ++k) t[k] = 0;
	for (uint64_t i = 0; i < n; ++i) {
		uint64_t b;
		memcpy(&b, &xs[i], 8);
		pg_fx_table_add(t, 1, pg_fx_widen(pg_fx_quant(b, s)), plain_add);
	}
	return pg_fx_table_double(t, 1, s);
}

extern "C" void fx_quant(double x, int s, uint64_t* w)
{
	uint64_t b;
	memcpy(&b, &x, 8);
	const pg_fx3 a = pg_fx_quant(b, s);
	w[0] = a.w0; w[1] = a.w1; w[2] = a.w2;
}

// Adds the 256-bit count w[0..4) into table words t[0..PG_FX_WORDS); returns
// whether the add marks the group present.
extern "C" int fx_table_add(uint64_t* t, const uint64_t* w)
{
	const pg_fx4 a = {w[0], w[1], w[2], w[3]};
	return pg_fx_table_add(t, 1, a, plain_add);
}

// The 256-bit count held by table words t[0..PG_FX_WORDS).
extern "C" void fx_table_count(const uint64_t* t, uint64_t* w)
{
	const pg_fx4 a = pg_fx_from_table(t, 1);
	w[0] = a.w0; w[1] = a.w1; w[2] = a.w2; w[3] = a.w3;
}

// The same for the four-word chained form of shared-memory tables.
extern "C" void fx_chain_add(uint64_t* t, const uint64_t* w)
{
	const pg_fx4 a = {w[0], w[1], w[2], w[3]};
	pg_fx_chain_add(t, 1, a, plain_add);
}

extern "C" void fx_chain_count(const uint64_t* t, uint64_t* w)
{
	const pg_fx4 a = pg_fx_from_chain(t, 1);
	w[0] = a.w0; w[1] = a.w1; w[2] = a.w2; w[3] = a.w3;
}

extern "C" double fx_double(const uint64_t* w, int s)
{
	const pg_fx4 a = {w[0], w[1], w[2], w[3]};
	return pg_fx_double4(a, s);
}

extern "C" uint64_t fx_special_bits(uint32_t flags) { return pg_fx_special_bits(flags); }
