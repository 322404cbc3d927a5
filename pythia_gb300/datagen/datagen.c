/*
 * Seeded synthetic relations for the Pythia GPU operator path.
 *
 * One generator feeds every consumer (GPU operators, the CPU oracle, the
 * reference engine's binary scans and the benchmarks), so all of them see the
 * same bytes. Rows use the reference's packed Page/Schema layout: a (long key,
 * long payload) tuple is 16 bytes, a (long key, dec value) tuple likewise
 * (schema.h:52-65, schema.inl:42-211).
 *
 * Published methods used (named, implemented here from their descriptions):
 *   - SplitMix64 (Steele, Lea, Flood 2014) to expand a 64-bit seed;
 *   - xoshiro256** (Blackman, Vigna 2018) as the stream generator;
 *   - Lemire's nearly-divisionless bounded integers (Lemire 2019);
 *   - Fisher-Yates / Durstenfeld shuffle for key permutations;
 *   - Zipf by rejection-inversion (Hormann, Derflinger 1996).
 *
 * Streams are cut into fixed chunks of 2^20 rows, each with its own
 * xoshiro state derived from (seed, chunk index), so the output does not
 * depend on how many threads produced it.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <pthread.h>

#define PGD_CHUNK (1u << 20)

static uint64_t splitmix64(uint64_t* s)
{
	uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

typedef struct { uint64_t s[4]; } xoshiro;

static inline uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static inline uint64_t xo_next(xoshiro* x)
{
	uint64_t* s = x->s;
	uint64_t result = rotl(s[1] * 5, 7) * 9;
	uint64_t t = s[1] << 17;
	s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
	s[2] ^= t; s[3] = rotl(s[3], 45);
	return result;
}

static void xo_seed(xoshiro* x, uint64_t seed, uint64_t stream)
{
	uint64_t sm = seed ^ (stream * 0xD1B54A32D192ED03ull);
	for (int i = 0; i < 4; ++i) x->s[i] = splitmix64(&sm);
}

/* Uniform in [0, range), range >= 1, unbiased (Lemire). */
static inline uint64_t bounded(xoshiro* x, uint64_t range)
{
	uint64_t r = xo_next(x);
	__uint128_t m = (__uint128_t) r * range;
	uint64_t lo = (uint64_t) m;
	if (lo < range) {
		uint64_t t = (0 - range) % range;
		while (lo < t) {
			r = xo_next(x);
			m = (__uint128_t) r * range;
			lo = (uint64_t) m;
		}
	}
	return (uint64_t) (m >> 64);
}

/* Uniform double in [0, 1) from the top 53 bits. */
static inline double unit53(xoshiro* x) { return (double) (xo_next(x) >> 11) * 0x1.0p-53; }

/* ---------------- Zipf, rejection-inversion ---------------- */
typedef struct {
	double s, hx1, hn, sx;
	uint64_t n;
} zipf_t;

/* (exp(t)-1)/t and log1p(t)/t with their limits at 0. */
static double h2(double t) { return fabs(t) > 1e-8 ? expm1(t) / t : 1.0 + t * 0.5 * (1.0 + t / 3.0); }
static double h1(double t) { return fabs(t) > 1e-8 ? log1p(t) / t : 1.0 - t * (0.5 - t / 3.0); }
static double zH(const zipf_t* z, double x) { double lx = log(x); return h2((1.0 - z->s) * lx) * lx; }
static double zHinv(const zipf_t* z, double u) { return exp(h1((1.0 - z->s) * u) * u); }
static double zh(const zipf_t* z, double x) { return exp(-z->s * log(x)); }

static void zipf_init(zipf_t* z, double s, uint64_t n)
{
	z->s = s; z->n = n;
	z->hx1 = zH(z, 1.5) - 1.0;
	z->hn = zH(z, (double) n + 0.5);
	z->sx = 2.0 - zHinv(z, zH(z, 2.5) - zh(z, 2.0));
}

/* Rank in [1, n] with P(k) proportional to k^-s. */
static uint64_t zipf_draw(const zipf_t* z, xoshiro* x)
{
	for (;;) {
		double u = z->hn + unit53(x) * (z->hx1 - z->hn);
		double xx = zHinv(z, u);
		double kd = floor(xx + 0.5);
		if (kd < 1.0) kd = 1.0;
		if (kd > (double) z->n) kd = (double) z->n;
		if (kd - xx <= z->sx || u >= zH(z, kd + 0.5) - zh(z, kd))
			return (uint64_t) kd;
	}
}

/* ---------------- chunked parallel driver ---------------- */
typedef void (*chunk_fn)(void* ctx, uint64_t chunk, uint64_t begin, uint64_t end);
typedef struct {
	chunk_fn fn; void* ctx; uint64_t n; uint64_t nchunks;
	int tid, nthreads;
} worker_arg;

static void* worker(void* p)
{
	worker_arg* a = (worker_arg*) p;
	for (uint64_t c = a->tid; c < a->nchunks; c += a->nthreads) {
		uint64_t b = c * PGD_CHUNK, e = b + PGD_CHUNK;
		if (e > a->n) e = a->n;
		a->fn(a->ctx, c, b, e);
	}
	return 0;
}

static void run_chunks(chunk_fn fn, void* ctx, uint64_t n, int threads)
{
	uint64_t nchunks = (n + PGD_CHUNK - 1) / PGD_CHUNK;
	if (threads < 1) threads = 1;
	if ((uint64_t) threads > nchunks) threads = nchunks ? (int) nchunks : 1;
	pthread_t th[256];
	worker_arg args[256];
	if (threads > 256) threads = 256;
	for (int t = 0; t < threads; ++t) {
		args[t].fn = fn; args[t].ctx = ctx; args[t].n = n; args[t].nchunks = nchunks;
		args[t].tid = t; args[t].nthreads = threads;
		if (t > 0) pthread_create(&th[t], 0, worker, &args[t]);
	}
	worker(&args[0]);
	for (int t = 1; t < threads; ++t) pthread_join(th[t], 0);
}

/* ---------------- relations ---------------- */
typedef struct {
	uint64_t seed;
	int64_t* rows;
	const int64_t* build;
	uint64_t nbuild, range;
	double s, vmax;
	zipf_t z;
} gen_ctx;

static void payload_chunk(void* p, uint64_t c, uint64_t b, uint64_t e)
{
	gen_ctx* g = (gen_ctx*) p; xoshiro x; xo_seed(&x, g->seed, c + 1);
	for (uint64_t i = b; i < e; ++i) g->rows[2 * i + 1] = (int64_t) (xo_next(&x) >> 33);
}

/*
 * Build relation: key = a random permutation of key_base .. key_base+n-1
 * (Durstenfeld shuffle), payload uniform in [0, 2^31).
 */
void pgd_gen_build(uint64_t seed, uint64_t n, int64_t key_base, int64_t* rows, int threads)
{
	xoshiro x; xo_seed(&x, seed, 0);
	for (uint64_t i = 0; i < n; ++i) rows[2 * i] = key_base + (int64_t) i;
	for (uint64_t i = n; i > 1; --i) {
		uint64_t j = bounded(&x, i);
		int64_t t = rows[2 * (i - 1)]; rows[2 * (i - 1)] = rows[2 * j]; rows[2 * j] = t;
	}
	gen_ctx g; memset(&g, 0, sizeof g); g.seed = seed; g.rows = rows;
	run_chunks(payload_chunk, &g, n, threads);
}

static void probe_uniform_chunk(void* p, uint64_t c, uint64_t b, uint64_t e)
{
	gen_ctx* g = (gen_ctx*) p; xoshiro x; xo_seed(&x, g->seed, c + 1);
	for (uint64_t i = b; i < e; ++i) {
		g->rows[2 * i] = g->build[2 * bounded(&x, g->nbuild)];
		g->rows[2 * i + 1] = (int64_t) (xo_next(&x) >> 33);
	}
}

/* Probe relation, foreign keys drawn uniformly over the build relation's keys. */
void pgd_gen_probe_uniform(uint64_t seed, uint64_t n, const int64_t* build, uint64_t nbuild,
		int64_t* rows, int threads)
{
	gen_ctx g; memset(&g, 0, sizeof g);
	g.seed = seed; g.rows = rows; g.build = build; g.nbuild = nbuild;
	run_chunks(probe_uniform_chunk, &g, n, threads);
}

static void probe_zipf_chunk(void* p, uint64_t c, uint64_t b, uint64_t e)
{
	gen_ctx* g = (gen_ctx*) p; xoshiro x; xo_seed(&x, g->seed, c + 1);
	for (uint64_t i = b; i < e; ++i) {
		uint64_t r = zipf_draw(&g->z, &x);
		g->rows[2 * i] = g->build[2 * (r - 1)];
		g->rows[2 * i + 1] = (int64_t) (xo_next(&x) >> 33);
	}
}

/*
 * Probe relation with Zipf(s) foreign keys: rank r maps to the key in build
 * row r-1. The build keys are a random permutation, so hot keys are spread
 * over the key domain rather than clustered at small values.
 */
void pgd_gen_probe_zipf(uint64_t seed, uint64_t n, double s, const int64_t* build, uint64_t nbuild,
		int64_t* rows, int threads)
{
	gen_ctx g; memset(&g, 0, sizeof g);
	g.seed = seed; g.rows = rows; g.build = build; g.nbuild = nbuild; g.s = s;
	zipf_init(&g.z, s, nbuild);
	run_chunks(probe_zipf_chunk, &g, n, threads);
}

static void uniform_keys_chunk(void* p, uint64_t c, uint64_t b, uint64_t e)
{
	gen_ctx* g = (gen_ctx*) p; xoshiro x; xo_seed(&x, g->seed, c + 1);
	for (uint64_t i = b; i < e; ++i) {
		g->rows[2 * i] = (int64_t) bounded(&x, g->range);
		g->rows[2 * i + 1] = (int64_t) (xo_next(&x) >> 33);
	}
}

/* (long key uniform in [0, range), long payload uniform in [0, 2^31)). */
void pgd_gen_uniform_keys(uint64_t seed, uint64_t n, uint64_t range, int64_t* rows, int threads)
{
	gen_ctx g; memset(&g, 0, sizeof g);
	g.seed = seed; g.rows = rows; g.range = range;
	run_chunks(uniform_keys_chunk, &g, n, threads);
}

static void groupby_chunk(void* p, uint64_t c, uint64_t b, uint64_t e)
{
	gen_ctx* g = (gen_ctx*) p; xoshiro x; xo_seed(&x, g->seed, c + 1);
	double* d = (double*) g->rows;
	for (uint64_t i = b; i < e; ++i) {
		g->rows[2 * i] = (int64_t) bounded(&x, g->range);
		d[2 * i + 1] = unit53(&x) * g->vmax;
	}
}

/* (long group key uniform in [0, groups), dec value uniform in [0, vmax)). */
void pgd_gen_groupby(uint64_t seed, uint64_t n, uint64_t groups, double vmax, void* rows, int threads)
{
	gen_ctx g; memset(&g, 0, sizeof g);
	g.seed = seed; g.rows = (int64_t*) rows; g.range = groups; g.vmax = vmax;
	run_chunks(groupby_chunk, &g, n, threads);
}

static void zipf_keys_chunk(void* p, uint64_t c, uint64_t b, uint64_t e)
{
	gen_ctx* g = (gen_ctx*) p; xoshiro x; xo_seed(&x, g->seed, c + 1);
	for (uint64_t i = b; i < e; ++i) {
		g->rows[2 * i] = (int64_t) zipf_draw(&g->z, &x) - 1;
		g->rows[2 * i + 1] = (int64_t) (xo_next(&x) >> 33);
	}
}

/* (long key = Zipf(s) rank - 1 over [0, range), long payload uniform). */
void pgd_gen_zipf_keys(uint64_t seed, uint64_t n, uint64_t range, double s, int64_t* rows, int threads)
{
	gen_ctx g; memset(&g, 0, sizeof g);
	g.seed = seed; g.rows = rows; g.range = range; g.s = s;
	zipf_init(&g.z, s, range);
	run_chunks(zipf_keys_chunk, &g, n, threads);
}

/* Raw xoshiro256** words for tests of the generator itself. */
void pgd_raw_words(uint64_t seed, uint64_t stream, uint64_t n, uint64_t* out)
{
	xoshiro x; xo_seed(&x, seed, stream);
	for (uint64_t i = 0; i < n; ++i) out[i] = xo_next(&x);
}

/* Bounded draws for tests of Lemire's method. */
void pgd_raw_bounded(uint64_t seed, uint64_t stream, uint64_t range, uint64_t n, uint64_t* out)
{
	xoshiro x; xo_seed(&x, seed, stream);
	for (uint64_t i = 0; i < n; ++i) out[i] = bounded(&x, range);
}
