// Host entry points over pythia_gb300/csrc/pg_fixsum.h for the Python test:
// quantisation of doubles to counts of units 2^s and the rounding of a
// 192-bit count back to a double, checked there against exact fractions.
#include "pg_fixsum.h"

extern "C" int fx_unit(int field, uint64_t n) { return pg_fx_unit(field, n); }

extern "C" int fx_field(double x)
{
	uint64_t b;
	memcpy(&b, &x, 8);
	return pg_fx_field(b);
}

// Sums xs[0..n) (all finite, fields <= the bound s was made from) as the GPU
// kernels do, in the given order; returns the double, the count in w[0..3).
extern "C" double fx_sum(const double* xs, uint64_t n, int s, uint64_t* w)
{
	pg_fx3 a = {0, 0, 0};
	for (uint64_t i = 0; i < n; ++i) {
		uint64_t b;
		memcpy(&b, &xs[i], 8);
		pg_fx_add(a, pg_fx_quant(b, s));
	}
	w[0] = a.w0; w[1] = a.w1; w[2] = a.w2;
	return pg_fx_double(a, s);
}

extern "C" void fx_quant(double x, int s, uint64_t* w)
{
	uint64_t b;
	memcpy(&b, &x, 8);
	const pg_fx3 a = pg_fx_quant(b, s);
	w[0] = a.w0; w[1] = a.w1; w[2] = a.w2;
}

extern "C" double fx_double(const uint64_t* w, int s)
{
	const pg_fx3 a = {w[0], w[1], w[2]};
	return pg_fx_double(a, s);
}

extern "C" uint64_t fx_special_bits(uint32_t flags) { return pg_fx_special_bits(flags); }
