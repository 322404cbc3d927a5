// Checks pg_add_err (integer rounding error of a double addition) bit for bit
// against Knuth's TwoSum on the host for random and edge-case operand pairs.
// Build: g++ -O2 -ffp-contract=off -I<repo>/pythia_gb300/csrc add_err_check.cpp
// Prints "ok <pairs>" or the first mismatches and exits 1.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include "pg_add_err.h"

static uint64_t s_state = 0x9E3779B97F4A7C15ull;
static uint64_t next64()
{
	uint64_t z = (s_state += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}
static double from_bits(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }
static uint64_t to_bits(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }

static double two_sum_err(double a, double b)
{
	volatile double s = a + b;
	volatile double bb = s - a;
	volatile double e = (a - (s - bb)) + (b - bb);
	return e;
}

static double pick(int kind)
{
	const uint64_t r = next64();
	switch (kind) {
	case 0: return from_bits(r);                                            // any bits
	case 1: return from_bits((r & 0x800FFFFFFFFFFFFFull) | ((uint64_t) (1000 + (r >> 52) % 48) << 52)); // similar exponents
	case 2: return from_bits(r & 0x800FFFFFFFFFFFFFull);                    // subnormals and zeros
	case 3: return std::ldexp((double) (int64_t) (r % 2001) - 1000.0, (int) ((r >> 20) % 120) - 60); // small integers scaled
	case 4: return from_bits((r & 0x8000000000000000ull) | ((uint64_t) ((r >> 52) % 2046 + 1) << 52)); // powers of two
	default: return (double) ((r >> 11) & ((1ull << 53) - 1)) * 0x1p-53 * 1e4;               // values in [0, 1e4)
	}
}

int main()
{
	long pairs = 0, bad = 0;
	for (int kind_a = 0; kind_a < 6; ++kind_a)
		for (int kind_b = 0; kind_b < 6; ++kind_b)
			for (int i = 0; i < 200000; ++i) {
				double a = pick(kind_a), b = pick(kind_b);
				if (i % 7 == 0) b = -a + pick(3) * 0x1p-40 * (std::isfinite(a) ? a : 1.0);   // cancellation
				if (i % 11 == 0) b = std::nextafter(-a, 0.0);
				if (!std::isfinite(a) || !std::isfinite(b) || !std::isfinite(a + b)) continue;
				if (std::fabs(a) > 0x1p1020 || std::fabs(b) > 0x1p1020) continue;       // TwoSum may overflow there
				const double want = two_sum_err(a, b);
				const double got = pg_add_err(a, b);
				++pairs;
				// Equal values (a signed zero compares equal to the other zero).
				if (!(want == got) && !(std::isnan(want) && std::isnan(got))) {
					if (bad < 10)
						printf("mismatch a=%a b=%a twosum=%a int=%a\n", a, b, want, got);
					++bad;
				}
			}
	// Ties to even: a = 2^53 + 2 (even), b = 1 -> RN(a+b) = 2^53 + 2 or +4?
	const double ties[][2] = {{0x1p53 + 2, 1.0}, {0x1p53, 1.0}, {0x1p53 + 4, 1.0}, {1.0, 0x1p-53},
		{1.0, 0x1p-54}, {1.0, -0x1p-54}, {1.0, 0x1.8p-53}, {-1.0, 0x1p-53}, {0x1p-1022, -0x1p-1074}};
	for (auto& t : ties) {
		const double want = two_sum_err(t[0], t[1]), got = pg_add_err(t[0], t[1]);
		++pairs;
		if (!(want == got)) { printf("tie mismatch a=%a b=%a twosum=%a int=%a\n", t[0], t[1], want, got); ++bad; }
	}
	if (bad) { printf("%ld of %ld pairs differ\n", bad, pairs); return 1; }
	printf("ok %ld\n", pairs);
	return 0;
}
