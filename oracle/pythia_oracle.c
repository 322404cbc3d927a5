/*
 * TEST INFRASTRUCTURE — the oracle. Not part of the product.
 *
 * Plain-C restatement of the reference Pythia operators on the GPU path
 * (see pythia_oracle.h). Used only by tests/, __graft_entry__.smoke() and
 * bench.py's CPU baseline and reference arm. Each function cites the
 * reference source it follows.
 */
#define _GNU_SOURCE
#include "pythia_oracle.h"
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <math.h>

/* ------------------------------------------------------------------ */
/* Hash functions: hash.h:51-479, hash.cpp:47-267                      */
/* ------------------------------------------------------------------ */

/* getlogarithm, hash.cpp:47-56: ceil(log2(k)), with getlogarithm(0) = 32. */
uint32_t or_getlogarithm(uint32_t k)
{
	--k;
	for (uint32_t i = 0; i < 32; ++i)
		if ((0x80000000u >> i) & k) return 32 - i;
	return 0;
}

/* The constructors of the HashFunction subclasses (hash.h:51-479) as
 * TupleHasher::create (hash.cpp:99-215) calls them. */
int or_hashfn_make(const or_hashcfg* c, or_hashfn* f)
{
	memset(f, 0, sizeof *f);
	f->fn = c->fn;
	if (c->fn == OR_FN_ALWAYSZERO) { f->k = 0; f->nbuckets = 1; return 0; }
	if (c->fn == OR_FN_TPCHQ1MAGIC) { f->k = 2; f->nbuckets = 4; return 0; }
	if (c->buckets == 0) return -1; /* HashFunction ctor throws, hash.cpp:61-64 */
	uint32_t lg = or_getlogarithm(c->buckets);
	switch (c->fn) {
	case OR_FN_BYTES: /* ByteHasher(buckets): _k = log2, hash.h:131-135 */
		f->k = lg; f->nbuckets = 1u << lg; break;
	case OR_FN_MODULO: /* _k = (1<<_k)-1 as mask, hash.h:273-277 */
	case OR_FN_TPCHORDERKEY:
	case OR_FN_WILLIS:
		f->k = (int64_t) ((1 << lg) - 1); f->nbuckets = (uint32_t) f->k + 1; break;
	case OR_FN_RANGE: /* RangeValueHasher, hash.h:238-258 */
		f->k = lg; f->min = c->min; f->max = c->max; f->nbuckets = 1u << lg; break;
	case OR_FN_EXACTRANGE: /* hash.h:444-479: _k = buckets, range = (max-min+k)/k */
		f->min = c->min; f->max = c->max; f->k = c->buckets;
		f->bucketrange = (f->max - f->min + f->k) / f->k;
		f->nbuckets = c->buckets; break;
	case OR_FN_PARAMMODULO: /* hash.h:301-338: mask <<= skipbits, _min = offset */
	case OR_FN_KNUTH:       /* hash.h:348-369 */
		f->k = (int64_t) ((1 << lg) - 1);
		f->skipbits = c->skipbits;
		f->k <<= c->skipbits;
		f->min = (int64_t) c->offset;
		f->nbuckets = (uint32_t) (f->k >> f->skipbits) + 1;
		break;
	default: return -1;
	}
	return 0;
}

/* ValueHasher::numericalize, hash.h:206-226: int32 sign-extends, int64 as is. */
static inline int64_t numericalize(const void* p, uint32_t size)
{
	if (size == 4) { int32_t v; memcpy(&v, p, 4); return v; }
	int64_t v; memcpy(&v, p, 8); return v;
}

uint32_t or_hash_value(const or_hashfn* f, const void* field, uint32_t size)
{
	switch (f->fn) {
	case OR_FN_BYTES: { /* FNV-1a-64 folded to _k bits, hash.h:137-170 */
		uint64_t h = 14695981039346656037ull;
		const signed char* p = (const signed char*) field;
		for (uint32_t i = 0; i < size; ++i) {
			h ^= (uint64_t) (int64_t) p[i];
			h += (h << 1) + (h << 4) + (h << 5) + (h << 7) + (h << 8) + (h << 40);
		}
		h = ((h >> f->k) ^ h) & ((1ull << f->k) - 1);
		return (uint32_t) h;
	}
	case OR_FN_TPCHQ1MAGIC: { /* hash.h:115-119 */
		uint32_t v; memcpy(&v, field, 4);
		return (((v >> 4) | (v >> 16)) & 0x1u) | ((v >> 1) & 0x2u);
	}
	case OR_FN_ALWAYSZERO: return 0;
	default: break;
	}
	int64_t v = numericalize(field, size);
	switch (f->fn) {
	case OR_FN_MODULO: return (uint32_t) (v & f->k); /* hash.h:279-282 */
	case OR_FN_RANGE: { /* hash.h:244-249 */
		int64_t val = v - f->min;
		val = (int64_t) ((uint64_t) val << f->k);
		return (uint32_t) (val / (f->max - f->min + 1));
	}
	case OR_FN_EXACTRANGE: return (uint32_t) ((v - f->min) / f->bucketrange); /* hash.h:457-461 */
	case OR_FN_PARAMMODULO: /* hash.h:317-320 */
		return (uint32_t) (((v - f->min) & f->k) >> f->skipbits);
	case OR_FN_KNUTH: /* hash.h:361-363: no offset subtraction */
		return (uint32_t) ((((uint64_t) v * 2654435761ull) & (uint64_t) f->k) >> f->skipbits);
	case OR_FN_TPCHORDERKEY: /* hash.h:389-391 */
		return (uint32_t) ((((v >> 2) & ~7LL) | (v & 7)) & f->k);
	case OR_FN_WILLIS: { /* hash.h:405-416 */
		int64_t l = v;
		l = (int64_t) (~(uint64_t) l + ((uint64_t) l << 21));
		l = l ^ (l >> 24);
		l = (int64_t) ((uint64_t) l + ((uint64_t) l << 3) + ((uint64_t) l << 8));
		l = l ^ (l >> 14);
		l = (int64_t) ((uint64_t) l + ((uint64_t) l << 2) + ((uint64_t) l << 4));
		l = l ^ (l >> 28);
		l = (int64_t) ((uint64_t) l + ((uint64_t) l << 31));
		l = (l > 0) ? l : (int64_t) (0 - (uint64_t) l);
		return (uint32_t) (l & f->k);
	}
	default: return 0;
	}
}

void or_hash_column(const or_hashfn* f, const void* rows, uint64_t n, uint32_t w,
		uint32_t off, uint32_t size, uint32_t* out)
{
	const char* r = (const char*) rows;
	for (uint64_t i = 0; i < n; ++i) out[i] = or_hash_value(f, r + i * w + off, size);
}

/* ExactRangeValueHasher::minimumforbucket, hash.h:463-468. */
int64_t or_exactrange_minimumforbucket(const or_hashfn* f, uint32_t bucket)
{
	if ((int64_t) bucket == f->k) return f->max + 1;
	return (int64_t) bucket * f->bucketrange + f->min;
}

/* ParameterizedModuloValueHasher::generate, hash.cpp:237-267. */
int or_parammodulo_generate(const or_hashfn* f, uint32_t passes, or_hashfn* out)
{
	if (f->fn != OR_FN_PARAMMODULO || passes == 0) return -1;
	uint32_t total = or_getlogarithm(f->nbuckets - 1);
	uint32_t per = total / passes;
	for (uint32_t i = 0; i + 1 < passes; ++i) {
		or_hashcfg c = { OR_FN_PARAMMODULO, 1u << per, 0, 0,
			f->skipbits + total - (i + 1) * per, (uint32_t) f->min };
		or_hashfn_make(&c, &out[i]);
	}
	uint32_t last = total - (passes - 1) * per;
	or_hashcfg c = { OR_FN_PARAMMODULO, 1u << last, 0, 0, f->skipbits, (uint32_t) f->min };
	or_hashfn_make(&c, &out[passes - 1]);
	return 0;
}

/* ------------------------------------------------------------------ */
/* Threads                                                             */
/* ------------------------------------------------------------------ */
typedef void* (*thr_fn)(void*);
static void run_threads(int T, thr_fn fn, void* args, size_t argsz)
{
	pthread_t th[512];
	if (T > 512) T = 512;
	for (int t = 1; t < T; ++t) pthread_create(&th[t], 0, fn, (char*) args + t * argsz);
	fn(args);
	for (int t = 1; t < T; ++t) pthread_join(th[t], 0);
}

static inline uint64_t slice_lo(uint64_t n, int t, int T) { return (uint64_t) ((__uint128_t) n * t / T); }

/* ------------------------------------------------------------------ */
/* Row-multiset digests (a checker utility, not a reference function)  */
/* ------------------------------------------------------------------ */
/* SplitMix64's finaliser (Steele, Lea and Flood, "Fast splittable
 * pseudorandom number generators", 2014). */
static inline uint64_t dg_mix(uint64_t z)
{
	z ^= z >> 30; z *= 0xBF58476D1CE4E5B9ull;
	z ^= z >> 27; z *= 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

/* Hash of one row: its 8-byte words (a short last word zero-filled) folded
 * in order, so two rows with the same words in other columns differ. */
static inline uint64_t dg_row_hash(const char* r, uint32_t w)
{
	uint64_t h = 0x243F6A8885A308D3ull ^ w;
	for (uint32_t o = 0; o < w; o += 8) {
		uint64_t x = 0;
		memcpy(&x, r + o, w - o < 8 ? w - o : 8);
		h = dg_mix(h ^ x) + 0x9E3779B97F4A7C15ull;
	}
	return h;
}

static inline void dg_add(or_digest* d, const char* r, uint32_t w)
{
	uint64_t x0 = 0, x1 = 0;
	memcpy(&x0, r, w < 8 ? w : 8);
	if (w > 8) memcpy(&x1, r + 8, w - 8 < 8 ? w - 8 : 8);
	d->n++; d->w0 += x0; d->w1 += x1; d->h += dg_row_hash(r, w);
}

static inline void dg_merge(or_digest* d, const or_digest* e)
{
	d->n += e->n; d->w0 += e->w0; d->w1 += e->w1; d->h += e->h;
}

typedef struct { const char* rows; uint64_t n; uint32_t w; int T, tid; or_digest d; } dg_arg;

static void* dg_thread(void* p)
{
	dg_arg* a = (dg_arg*) p;
	uint64_t lo = slice_lo(a->n, a->tid, a->T), hi = slice_lo(a->n, a->tid + 1, a->T);
	for (uint64_t i = lo; i < hi; ++i) dg_add(&a->d, a->rows + i * a->w, a->w);
	return 0;
}

void or_rows_digest(const void* rows, uint64_t n, uint32_t w, int threads, or_digest* d)
{
	if (threads < 1) threads = 1;
	dg_arg* args = (dg_arg*) calloc(threads, sizeof(dg_arg));
	for (int t = 0; t < threads; ++t) {
		args[t].rows = (const char*) rows; args[t].n = n; args[t].w = w; args[t].T = threads; args[t].tid = t;
	}
	run_threads(threads, dg_thread, args, sizeof(dg_arg));
	memset(d, 0, sizeof *d);
	for (int t = 0; t < threads; ++t) dg_merge(d, &args[t].d);
	free(args);
}

/* ------------------------------------------------------------------ */
/* Chained-bucket hash table: util/hashtable.{h,cpp}                   */
/* ------------------------------------------------------------------ */
/* BucketHeader {Lock (1 byte TAS), unsigned short used, BucketHeader* next},
 * util/hashtable.h:244-267; a bucket is the header followed by bucksize
 * bytes of tuples; overflow chains a freshly allocated bucket
 * (util/hashtable.cpp:230-273). */
typedef struct bhdr { volatile char lock; uint16_t used; struct bhdr* next; } bhdr;

typedef struct {
	char* mem; uint32_t nbuckets, bucksize, tuplesize;
} chtable;

typedef struct { char* cur; size_t left; void** blocks; int nblocks, cap; } arena;

static void* arena_alloc(arena* a, size_t sz)
{
	sz = (sz + 15) & ~(size_t) 15;
	if (a->left < sz) {
		size_t bs = sz > (1u << 20) ? sz : (1u << 20);
		if (a->nblocks == a->cap) {
			a->cap = a->cap ? 2 * a->cap : 16;
			a->blocks = (void**) realloc(a->blocks, a->cap * sizeof(void*));
		}
		a->cur = (char*) malloc(bs); a->left = bs;
		a->blocks[a->nblocks++] = a->cur;
	}
	void* r = a->cur; a->cur += sz; a->left -= sz; return r;
}

static void arena_free(arena* a)
{
	for (int i = 0; i < a->nblocks; ++i) free(a->blocks[i]);
	free(a->blocks); memset(a, 0, sizeof *a);
}

static inline bhdr* ch_bucket(const chtable* t, uint32_t b)
{
	return (bhdr*) (t->mem + (size_t) b * (sizeof(bhdr) + t->bucksize));
}

static int ch_init(chtable* t, uint32_t nbuckets, uint32_t bucksize, uint32_t tuplesize)
{
	t->nbuckets = nbuckets; t->bucksize = bucksize; t->tuplesize = tuplesize;
	t->mem = (char*) calloc((size_t) nbuckets, sizeof(bhdr) + bucksize);
	return t->mem ? 0 : -1;
}

/* HashTable::allocate, util/hashtable.cpp:230-273. */
static void* ch_allocate(chtable* t, uint32_t b, arena* a)
{
	bhdr* last = 0;
	for (bhdr* h = ch_bucket(t, b); h; h = h->next) {
		if (h->used + t->tuplesize <= t->bucksize) {
			void* r = (char*) h + sizeof(bhdr) + h->used;
			h->used += t->tuplesize;
			return r;
		}
		last = h;
	}
	bhdr* nb = (bhdr*) arena_alloc(a, sizeof(bhdr) + t->bucksize);
	nb->lock = 0; nb->used = t->tuplesize; nb->next = 0;
	last->next = nb;
	return (char*) nb + sizeof(bhdr);
}

/* HashTable::atomicAllocate, util/hashtable.h:99-108 (bucket TAS spinlock). */
static void* ch_atomic_allocate(chtable* t, uint32_t b, arena* a)
{
	bhdr* h = ch_bucket(t, b);
	while (__atomic_test_and_set((void*) &h->lock, __ATOMIC_ACQUIRE)) { }
	void* r = ch_allocate(t, b, a);
	__atomic_clear((void*) &h->lock, __ATOMIC_RELEASE);
	return r;
}

/* ------------------------------------------------------------------ */
/* Hash join: operators/join.cpp:273-675                               */
/* ------------------------------------------------------------------ */
typedef struct {
	char* data; size_t used, cap;
} growbuf;

static void gb_push(growbuf* g, const void* p, size_t n)
{
	if (g->used + n > g->cap) {
		size_t nc = g->cap ? g->cap * 2 : (1u << 16);
		while (nc < g->used + n) nc *= 2;
		g->data = (char*) realloc(g->data, nc); g->cap = nc;
	}
	memcpy(g->data + g->used, p, n); g->used += n;
}

static inline int keys_equal(const void* a, uint32_t as, const void* b, uint32_t bs)
{
	return numericalize(a, as) == numericalize(b, bs);
}

typedef struct {
	/* shared */
	const char *R, *S; uint64_t nR, nS; uint32_t wR, wS, bkoff, bkbytes, pkoff, pkbytes;
	or_hashfn fn; chtable* ht; const or_col* proj; int nproj;
	uint32_t sw, ow; int sum_col; int T; pthread_barrier_t* bar;
	uint32_t* bproj_off; uint32_t nbproj; /* build-projected source offsets/bytes */
	uint32_t* bproj_bytes;
	int materialise, digest;
	uint32_t page_bytes;   /* > 0: rows go to one reused output page per thread */
	/* per thread */
	int tid; arena ar; growbuf out; uint64_t nout; int64_t sum; or_digest dg;
	char* page; uint32_t page_used; uint64_t pages;
} hj_arg;

static int64_t col_as_i64(const char* p, uint32_t bytes)
{
	if (bytes == 4) { int32_t v; memcpy(&v, p, 4); return v; }
	int64_t v; memcpy(&v, p, 8); return v;
}

static void* hj_thread(void* p)
{
	hj_arg* a = (hj_arg*) p;
	/* buildFromPage, join.cpp:641-667: hash the build key, atomicAllocate,
	 * write the key then each build-projected column into the sbuild tuple. */
	uint64_t lo = slice_lo(a->nR, a->tid, a->T), hi = slice_lo(a->nR, a->tid + 1, a->T);
	for (uint64_t i = lo; i < hi; ++i) {
		const char* tup = a->R + i * a->wR;
		uint32_t h = or_hash_value(&a->fn, tup + a->bkoff, a->bkbytes);
		char* dst = (char*) ch_atomic_allocate(a->ht, h, &a->ar);
		memcpy(dst, tup + a->bkoff, a->bkbytes);
		uint32_t o = a->bkbytes;
		for (uint32_t j = 0; j < a->nbproj; ++j) {
			memcpy(dst + o, tup + a->bproj_off[j], a->bproj_bytes[j]);
			o += a->bproj_bytes[j];
		}
	}
	/* Group barrier before probing, join.cpp:434. */
	pthread_barrier_wait(a->bar);
	/* getNext probe loop, join.cpp:503-562: hash the probe key, walk the
	 * bucket chain, compare keys, constructOutputTuple (join.cpp:475-501). */
	lo = slice_lo(a->nS, a->tid, a->T); hi = slice_lo(a->nS, a->tid + 1, a->T);
	char rowbuf[1024];
	for (uint64_t i = lo; i < hi; ++i) {
		const char* ptup = a->S + i * a->wS;
		uint32_t h = or_hash_value(&a->fn, ptup + a->pkoff, a->pkbytes);
		for (bhdr* bh = ch_bucket(a->ht, h); bh; bh = bh->next) {
			const char* b = (const char*) bh + sizeof(bhdr);
			for (uint32_t u = 0; u < bh->used; u += a->sw, b += a->sw) {
				if (!keys_equal(b, a->bkbytes, ptup + a->pkoff, a->pkbytes)) continue;
				/* With pages, constructOutputTuple writes straight into the
				 * thread's output page, which is handed on (here: reused)
				 * once the next row would not fit (join.cpp:510-545). */
				char* row = a->page ? a->page + a->page_used : rowbuf;
				uint32_t o = 0, battr = a->bkbytes;
				for (int j = 0; j < a->nproj; ++j) {
					const or_col* c = &a->proj[j];
					if (c->side == 0) { memcpy(row + o, b + battr, c->bytes); battr += c->bytes; }
					else memcpy(row + o, ptup + c->off, c->bytes);
					if (j == a->sum_col) a->sum += col_as_i64(row + o, c->bytes);
					o += c->bytes;
				}
				a->nout++;
				if (a->materialise) gb_push(&a->out, row, a->ow);
				if (a->digest) dg_add(&a->dg, row, a->ow);
				if (a->page) {
					a->page_used += a->ow;
					if (a->page_used + a->ow > a->page_bytes) { a->page_used = 0; a->pages++; }
				}
			}
		}
	}
	return 0;
}

static int hashjoin_run(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_hashcfg* hash, uint32_t tuplesperbucket,
		const or_col* proj, int nproj, void* out, uint64_t out_cap,
		int sum_col, int threads, or_join_result* res, or_digest* dg, uint32_t page_bytes);

int or_hashjoin(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_hashcfg* hash, uint32_t tuplesperbucket,
		const or_col* proj, int nproj, void* out, uint64_t out_cap,
		int sum_col, int threads, or_join_result* res)
{
	return hashjoin_run(R, nR, wR, bkoff, bkbytes, S, nS, wS, pkoff, pkbytes, hash, tuplesperbucket,
			proj, nproj, out, out_cap, sum_col, threads, res, 0, 0);
}

int or_hashjoin_paged(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_hashcfg* hash, uint32_t tuplesperbucket,
		const or_col* proj, int nproj, uint32_t page_bytes,
		int sum_col, int threads, or_join_result* res)
{
	if (page_bytes == 0) return -1;
	return hashjoin_run(R, nR, wR, bkoff, bkbytes, S, nS, wS, pkoff, pkbytes, hash, tuplesperbucket,
			proj, nproj, 0, 0, sum_col, threads, res, 0, page_bytes);
}

int or_hashjoin_digest(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_hashcfg* hash, uint32_t tuplesperbucket,
		const or_col* proj, int nproj, int threads, or_digest* dg)
{
	or_join_result res;
	memset(dg, 0, sizeof *dg);
	return hashjoin_run(R, nR, wR, bkoff, bkbytes, S, nS, wS, pkoff, pkbytes, hash, tuplesperbucket,
			proj, nproj, 0, 0, -1, threads, &res, dg, 0);
}

static int hashjoin_run(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_hashcfg* hash, uint32_t tuplesperbucket,
		const or_col* proj, int nproj, void* out, uint64_t out_cap,
		int sum_col, int threads, or_join_result* res, or_digest* dg, uint32_t page_bytes)
{
	or_hashfn fn;
	if (or_hashfn_make(hash, &fn)) return -1;
	if (threads < 1) threads = 1;
	/* sbuild = (key, build-projected columns), join.cpp:287-297. */
	uint32_t sw = bkbytes, ow = 0, nb = 0;
	uint32_t boff[64], bbytes[64];
	for (int j = 0; j < nproj; ++j) {
		ow += proj[j].bytes;
		if (proj[j].side == 0) { sw += proj[j].bytes; boff[nb] = proj[j].off; bbytes[nb++] = proj[j].bytes; }
	}
	if (ow > 1024 || nb > 64 || (page_bytes && page_bytes < ow)) return -1;
	chtable ht;
	if (ch_init(&ht, fn.nbuckets, tuplesperbucket * sw, sw)) return -1;
	pthread_barrier_t bar; pthread_barrier_init(&bar, 0, threads);
	hj_arg* args = (hj_arg*) calloc(threads, sizeof(hj_arg));
	for (int t = 0; t < threads; ++t) {
		hj_arg* a = &args[t];
		a->R = (const char*) R; a->S = (const char*) S; a->nR = nR; a->nS = nS;
		a->wR = wR; a->wS = wS; a->bkoff = bkoff; a->bkbytes = bkbytes;
		a->pkoff = pkoff; a->pkbytes = pkbytes; a->fn = fn; a->ht = &ht;
		a->proj = proj; a->nproj = nproj; a->sw = sw; a->ow = ow; a->sum_col = sum_col;
		a->T = threads; a->bar = &bar; a->bproj_off = boff; a->bproj_bytes = bbytes;
		a->nbproj = nb; a->materialise = out != 0; a->digest = dg != 0; a->tid = t;
		a->page_bytes = page_bytes;
		a->page = page_bytes ? (char*) malloc(page_bytes) : 0;
	}
	run_threads(threads, hj_thread, args, sizeof(hj_arg));
	uint64_t total = 0, written = 0; int64_t sum = 0;
	for (int t = 0; t < threads; ++t) {
		hj_arg* a = &args[t];
		total += a->nout; sum = (int64_t) ((uint64_t) sum + (uint64_t) a->sum);
		if (dg) dg_merge(dg, &a->dg);
		free(a->page);
		if (out) {
			uint64_t rows = a->out.used / ow;
			uint64_t take = rows;
			if (written + take > out_cap) take = out_cap > written ? out_cap - written : 0;
			memcpy((char*) out + written * ow, a->out.data, take * ow);
			written += take;
		}
		free(a->out.data); arena_free(&a->ar);
	}
	free(args); free(ht.mem); pthread_barrier_destroy(&bar);
	res->n_out = total; res->sum = sum;
	return 0;
}

/* ------------------------------------------------------------------ */
/* Partition: operators/partition.cpp:166-359                          */
/* ------------------------------------------------------------------ */
typedef struct {
	const char* in; uint64_t n; uint32_t w, koff, kbytes; or_hashfn fn;
	char* out; uint64_t* hist; /* [T][nb] */ int T, tid; uint32_t nb;
	pthread_barrier_t* bar; uint64_t* offsets;
} part_arg;

static void* part_thread(void* p)
{
	part_arg* a = (part_arg*) p;
	uint64_t lo = slice_lo(a->n, a->tid, a->T), hi = slice_lo(a->n, a->tid + 1, a->T);
	uint64_t* my = a->hist + (size_t) a->tid * a->nb;
	/* copySourceIntoPageAndPopulateHistogram, partition.cpp:166-200. */
	for (uint64_t i = lo; i < hi; ++i) {
		uint32_t h = or_hash_value(&a->fn, a->in + i * a->w + a->koff, a->kbytes);
		my[h]++;
	}
	pthread_barrier_wait(a->bar);
	/* Prefix over threads per partition, partition.cpp:292-307; thread 0
	 * also lays the partitions out back to back. */
	if (a->tid == 0) {
		uint64_t run = 0;
		for (uint32_t b = 0; b < a->nb; ++b) {
			a->offsets[b] = run;
			for (int t = 0; t < a->T; ++t) {
				uint64_t c = a->hist[(size_t) t * a->nb + b];
				a->hist[(size_t) t * a->nb + b] = run;
				run += c;
			}
		}
		a->offsets[a->nb] = run;
	}
	pthread_barrier_wait(a->bar);
	/* repartition, partition.cpp:250-268: stable scatter. */
	for (uint64_t i = lo; i < hi; ++i) {
		const char* tup = a->in + i * a->w;
		uint32_t h = or_hash_value(&a->fn, tup + a->koff, a->kbytes);
		memcpy(a->out + my[h] * a->w, tup, a->w);
		my[h]++;
	}
	return 0;
}

int or_partition(const void* in, uint64_t n, uint32_t w, uint32_t koff, uint32_t kbytes,
		const or_hashcfg* hash, void* out, uint64_t* offsets, int threads)
{
	or_hashfn fn;
	if (or_hashfn_make(hash, &fn)) return -1;
	/* Every tuple must land in [0, buckets) (partition.cpp:184-185, dbgassert). */
	const char* r = (const char*) in;
	for (uint64_t i = 0; i < n; ++i)
		if (or_hash_value(&fn, r + i * w + koff, kbytes) >= fn.nbuckets) return -2;
	if (threads < 1) threads = 1;
	pthread_barrier_t bar; pthread_barrier_init(&bar, 0, threads);
	uint64_t* hist = (uint64_t*) calloc((size_t) threads * fn.nbuckets, sizeof(uint64_t));
	part_arg* args = (part_arg*) calloc(threads, sizeof(part_arg));
	for (int t = 0; t < threads; ++t) {
		part_arg* a = &args[t];
		a->in = r; a->n = n; a->w = w; a->koff = koff; a->kbytes = kbytes; a->fn = fn;
		a->out = (char*) out; a->hist = hist; a->T = threads; a->tid = t; a->nb = fn.nbuckets;
		a->bar = &bar; a->offsets = offsets;
	}
	run_threads(threads, part_thread, args, sizeof(part_arg));
	free(args); free(hist); pthread_barrier_destroy(&bar);
	return 0;
}

/* ------------------------------------------------------------------ */
/* Aggregation: operators/genericaggregate.cpp:240-487,                */
/* aggregatesum.cpp:53-107, aggregatecount.cpp:37-52                   */
/* ------------------------------------------------------------------ */
typedef struct {
	const char* in; uint64_t n; uint32_t w, koff, kbytes, voff; int has_key, vtype, agg;
	or_hashfn fn; uint32_t gw, aw; int T, tid;
	chtable ht; arena ar;
} agg_arg;

static void agg_fold(char* acc, const char* tup, int vtype, int agg, int start)
{
	if (agg == OR_AGG_COUNT) { /* foldstart = 1, fold ++ */
		int64_t c; if (start) c = 1; else { memcpy(&c, acc, 8); c++; }
		memcpy(acc, &c, 8); return;
	}
	if (vtype == OR_VAL_INT) {
		int32_t v, s; memcpy(&v, tup, 4);
		if (start) s = v; else { memcpy(&s, acc, 4); s = (int32_t) ((uint32_t) s + (uint32_t) v); }
		memcpy(acc, &s, 4);
	} else if (vtype == OR_VAL_LONG) {
		int64_t v, s; memcpy(&v, tup, 8);
		if (start) s = v; else { memcpy(&s, acc, 8); s = (int64_t) ((uint64_t) s + (uint64_t) v); }
		memcpy(acc, &s, 8);
	} else {
		double v, s; memcpy(&v, tup, 8);
		if (start) s = v; else { memcpy(&s, acc, 8); s += v; }
		memcpy(acc, &s, 8);
	}
}

/* Merge an existing partial (stage two): int sums add, counts add. */
static void agg_merge(char* acc, const char* part, int vtype, int agg, int start)
{
	if (start) { memcpy(acc, part, (agg == OR_AGG_SUM && vtype == OR_VAL_INT) ? 4 : 8); return; }
	if (agg == OR_AGG_COUNT || vtype == OR_VAL_LONG) {
		int64_t a, b; memcpy(&a, acc, 8); memcpy(&b, part, 8);
		a = (int64_t) ((uint64_t) a + (uint64_t) b); memcpy(acc, &a, 8);
	} else if (vtype == OR_VAL_INT) {
		int32_t a, b; memcpy(&a, acc, 4); memcpy(&b, part, 4);
		a = (int32_t) ((uint32_t) a + (uint32_t) b); memcpy(acc, &a, 4);
	} else {
		double a, b; memcpy(&a, acc, 8); memcpy(&b, part, 8); a += b; memcpy(acc, &a, 8);
	}
}

/* remember, genericaggregate.cpp:240-282: walk the chain of the key's bucket,
 * fold on a match, else allocate + copy key + foldstart. Tables are
 * thread-local (the default ThreadLocal mode). */
static char* agg_find_or_insert(agg_arg* a, const char* key, int* fresh)
{
	uint32_t h = a->has_key ? or_hash_value(&a->fn, key, a->kbytes) : 0;
	for (bhdr* bh = ch_bucket(&a->ht, h); bh; bh = bh->next) {
		char* t = (char*) bh + sizeof(bhdr);
		for (uint32_t u = 0; u < bh->used; u += a->ht.tuplesize, t += a->ht.tuplesize)
			if (!a->has_key || memcmp(t, key, a->kbytes) == 0) { *fresh = 0; return t; }
	}
	char* t = (char*) ch_allocate(&a->ht, h, &a->ar);
	if (a->has_key) memcpy(t, key, a->kbytes);
	*fresh = 1;
	return t;
}

static void* agg_thread(void* p)
{
	agg_arg* a = (agg_arg*) p;
	uint64_t lo = slice_lo(a->n, a->tid, a->T), hi = slice_lo(a->n, a->tid + 1, a->T);
	for (uint64_t i = lo; i < hi; ++i) {
		const char* tup = a->in + i * a->w;
		int fresh;
		char* t = agg_find_or_insert(a, tup + a->koff, &fresh);
		agg_fold(t + a->gw, tup + a->voff, a->vtype, a->agg, fresh);
	}
	return 0;
}

int or_groupby(const void* in, uint64_t n, uint32_t w, int has_key, uint32_t koff, uint32_t kbytes,
		uint32_t voff, int vtype, int agg, const or_hashcfg* hash,
		void* out, uint64_t out_cap, uint64_t* ngroups, int threads)
{
	or_hashcfg zero = { OR_FN_ALWAYSZERO, 1, 0, 0, 0, 0 };
	or_hashfn fn;
	if (or_hashfn_make(has_key ? hash : &zero, &fn)) return -1;
	if (threads < 1) threads = 1;
	uint32_t gw = has_key ? kbytes : 0;
	uint32_t aw = (agg == OR_AGG_SUM && vtype == OR_VAL_INT) ? 4 : 8;
	uint32_t tw = gw + aw;
	agg_arg* args = (agg_arg*) calloc(threads + 1, sizeof(agg_arg));
	for (int t = 0; t <= threads; ++t) {
		agg_arg* a = &args[t];
		a->in = (const char*) in; a->n = n; a->w = w; a->koff = koff; a->kbytes = kbytes;
		a->voff = voff; a->has_key = has_key; a->vtype = vtype; a->agg = agg; a->fn = fn;
		a->gw = gw; a->aw = aw; a->T = threads; a->tid = t;
		/* bucket holds four tuples, genericaggregate.cpp:181-186 */
		if (ch_init(&a->ht, fn.nbuckets, 4 * tw, tw)) return -1;
	}
	run_threads(threads, agg_thread, args, sizeof(agg_arg));
	/* Stage two (merge + second aggregate over the partials), as the
	 * reference's two-stage plans do: partials merged in thread order. */
	agg_arg* fin = &args[threads];
	for (int t = 0; t < threads; ++t) {
		agg_arg* a = &args[t];
		for (uint32_t b = 0; b < a->ht.nbuckets; ++b)
			for (bhdr* bh = ch_bucket(&a->ht, b); bh; bh = bh->next) {
				char* tp = (char*) bh + sizeof(bhdr);
				for (uint32_t u = 0; u < bh->used; u += tw, tp += tw) {
					int fresh;
					char* d = agg_find_or_insert(fin, tp, &fresh);
					agg_merge(d + gw, tp + gw, vtype, agg, fresh);
				}
			}
	}
	/* getNext, genericaggregate.cpp:419-487: emit bucket by bucket. */
	uint64_t g = 0;
	for (uint32_t b = 0; b < fin->ht.nbuckets; ++b)
		for (bhdr* bh = ch_bucket(&fin->ht, b); bh; bh = bh->next) {
			char* tp = (char*) bh + sizeof(bhdr);
			for (uint32_t u = 0; u < bh->used; u += tw, tp += tw) {
				if (g < out_cap) memcpy((char*) out + g * tw, tp, tw);
				g++;
			}
		}
	*ngroups = g;
	for (int t = 0; t <= threads; ++t) { free(args[t].ht.mem); arena_free(&args[t].ar); }
	free(args);
	return 0;
}

/* Exactly rounded sum of doubles (Shewchuk's adaptive-precision partials,
 * "Adaptive Precision Floating-Point Arithmetic", 1997, the method behind
 * Python's math.fsum), including its final round-half-even correction. */
double or_fsum(const double* x, uint64_t n, uint64_t stride)
{
	size_t cap = 32, np = 0;
	double* p = (double*) malloc(cap * sizeof(double));
	for (uint64_t i = 0; i < n; ++i) {
		double v = x[i * stride];
		size_t k = 0;
		for (size_t j = 0; j < np; ++j) {
			double y = p[j];
			if (fabs(v) < fabs(y)) { double t = v; v = y; y = t; }
			double hi = v + y;
			double lo = y - (hi - v);
			if (lo != 0.0) p[k++] = lo;
			v = hi;
		}
		if (k == cap) { cap *= 2; p = (double*) realloc(p, cap * sizeof(double)); }
		p[k++] = v; np = k;
	}
	double hi = 0.0;
	if (np > 0) {
		size_t j = np - 1;
		hi = p[j];
		double lo = 0.0;
		while (j > 0) {
			double v = hi; double y = p[--j];
			hi = v + y;
			double yr = hi - v;
			lo = y - yr;
			if (lo != 0.0) break;
		}
		if (j > 0 && ((lo < 0.0 && p[j - 1] < 0.0) || (lo > 0.0 && p[j - 1] > 0.0))) {
			double y = lo * 2.0;
			double v = hi + y;
			double yr = v - hi;
			if (y == yr) hi = v;
		}
	}
	free(p);
	return hi;
}

/* ------------------------------------------------------------------ */
/* Sorting (TupleBuffer::sort<KeyT>, util/buffer.inl:135-292)          */
/* ------------------------------------------------------------------ */
typedef struct { int64_t key; uint64_t idx; } kidx;

/* Stable bottom-up merge sort on (key, index) pairs. */
static void kidx_sort(kidx* a, uint64_t n)
{
	kidx* tmp = (kidx*) malloc((n ? n : 1) * sizeof(kidx));
	kidx *src = a, *dst = tmp;
	for (uint64_t width = 1; width < n; width *= 2) {
		for (uint64_t lo = 0; lo < n; lo += 2 * width) {
			uint64_t mid = lo + width < n ? lo + width : n;
			uint64_t hi = lo + 2 * width < n ? lo + 2 * width : n;
			uint64_t i = lo, j = mid, k = lo;
			while (i < mid && j < hi) dst[k++] = (src[j].key < src[i].key) ? src[j++] : src[i++];
			while (i < mid) dst[k++] = src[i++];
			while (j < hi) dst[k++] = src[j++];
		}
		kidx* t = src; src = dst; dst = t;
	}
	if (src != a) memcpy(a, src, n * sizeof(kidx));
	free(tmp);
}

static kidx* sorted_index(const char* in, uint64_t n, uint32_t w, uint32_t koff, uint32_t kbytes)
{
	kidx* k = (kidx*) malloc((n ? n : 1) * sizeof(kidx));
	for (uint64_t i = 0; i < n; ++i) { k[i].key = numericalize(in + i * w + koff, kbytes); k[i].idx = i; }
	kidx_sort(k, n);
	return k;
}

/* Sorted by key (signed compare, as the CtInt/CtLong comparators do);
 * ties keep input order (std::sort leaves their order unspecified). */
int or_sort(const void* in, uint64_t n, uint32_t w, uint32_t koff, uint32_t kbytes, void* out)
{
	const char* r = (const char*) in;
	kidx* k = sorted_index(r, n, w, koff, kbytes);
	for (uint64_t i = 0; i < n; ++i) memcpy((char*) out + i * w, r + k[i].idx * w, w);
	free(k);
	return 0;
}

int or_groupby_exact(const void* in, uint64_t n, uint32_t w, int has_key, uint32_t koff,
		uint32_t kbytes, uint32_t voff, void* out, uint64_t out_cap, uint64_t* ngroups)
{
	const char* r = (const char*) in;
	kidx* k;
	if (has_key) k = sorted_index(r, n, w, koff, kbytes);
	else {
		k = (kidx*) malloc((n ? n : 1) * sizeof(kidx));
		for (uint64_t i = 0; i < n; ++i) { k[i].key = 0; k[i].idx = i; }
	}
	double* vals = (double*) malloc((n ? n : 1) * sizeof(double));
	uint32_t gw = has_key ? kbytes : 0, tw = gw + 8;
	uint64_t g = 0, i = 0;
	while (i < n) {
		uint64_t j = i;
		while (j < n && k[j].key == k[i].key) { memcpy(&vals[j - i], r + k[j].idx * w + voff, 8); ++j; }
		if (g < out_cap) {
			char* o = (char*) out + g * tw;
			if (has_key) memcpy(o, r + k[i].idx * w + koff, kbytes);
			double s = or_fsum(vals, j - i, 1);
			memcpy(o + gw, &s, 8);
		}
		g++; i = j;
	}
	*ngroups = g;
	free(k); free(vals);
	return 0;
}

/* ------------------------------------------------------------------ */
/* Sort-merge / MPSM join: operators/join.cpp:945-1371                 */
/* ------------------------------------------------------------------ */
typedef struct {
	const char *R, *S; uint64_t nR, nS; uint32_t wR, wS, bkoff, bkbytes, pkoff, pkbytes;
	const or_col* proj; int nproj; uint32_t ow; int sum_col, T, tid, materialise, digest;
	kidx** rruns; kidx** sruns; uint64_t *rlen, *slen; uint64_t *rlo, *slo;
	pthread_barrier_t* bar;
	growbuf out; uint64_t nout; int64_t sum; or_digest dg;
} mj_arg;

static void* mj_thread(void* p)
{
	mj_arg* a = (mj_arg*) p;
	/* BufferAndSort, join.cpp:945-996: each thread sorts its build run and
	 * its probe run. */
	uint64_t rlo = slice_lo(a->nR, a->tid, a->T), rhi = slice_lo(a->nR, a->tid + 1, a->T);
	uint64_t slo = slice_lo(a->nS, a->tid, a->T), shi = slice_lo(a->nS, a->tid + 1, a->T);
	a->rruns[a->tid] = sorted_index(a->R + rlo * a->wR, rhi - rlo, a->wR, a->bkoff, a->bkbytes);
	a->sruns[a->tid] = sorted_index(a->S + slo * a->wS, shi - slo, a->wS, a->pkoff, a->pkbytes);
	a->rlen[a->tid] = rhi - rlo; a->slen[a->tid] = shi - slo;
	a->rlo[a->tid] = rlo; a->slo[a->tid] = slo;
	pthread_barrier_wait(a->bar);
	/* OldMPSMJoinOp::getNext, join.cpp:1245-1371: merge this thread's build
	 * run against every probe run in turn; equal-key groups produce their
	 * cartesian product. */
	kidx* rr = a->rruns[a->tid]; uint64_t nr = a->rlen[a->tid];
	const char* rbase = a->R + a->rlo[a->tid] * a->wR;
	char row[1024];
	for (int s = 0; s < a->T; ++s) {
		kidx* sr = a->sruns[s]; uint64_t ns = a->slen[s];
		const char* sbase = a->S + a->slo[s] * a->wS;
		uint64_t i = 0, j = 0;
		while (i < nr && j < ns) {
			if (rr[i].key < sr[j].key) { ++i; continue; }
			if (sr[j].key < rr[i].key) { ++j; continue; }
			uint64_t i1 = i, j1 = j;
			while (i1 < nr && rr[i1].key == rr[i].key) ++i1;
			while (j1 < ns && sr[j1].key == sr[j].key) ++j1;
			for (uint64_t y = j; y < j1; ++y)
				for (uint64_t x = i; x < i1; ++x) {
					const char* bt = rbase + rr[x].idx * a->wR;
					const char* pt = sbase + sr[y].idx * a->wS;
					uint32_t o = 0;
					for (int c = 0; c < a->nproj; ++c) {
						const or_col* col = &a->proj[c];
						memcpy(row + o, (col->side == 0 ? bt : pt) + col->off, col->bytes);
						if (c == a->sum_col) a->sum += col_as_i64(row + o, col->bytes);
						o += col->bytes;
					}
					a->nout++;
					if (a->materialise) gb_push(&a->out, row, a->ow);
					if (a->digest) dg_add(&a->dg, row, a->ow);
				}
			i = i1; j = j1;
		}
	}
	return 0;
}

static int mergejoin_run(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_col* proj, int nproj, void* out, uint64_t out_cap,
		int sum_col, int threads, or_join_result* res, or_digest* dg);

int or_mergejoin(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_col* proj, int nproj, void* out, uint64_t out_cap,
		int sum_col, int threads, or_join_result* res)
{
	return mergejoin_run(R, nR, wR, bkoff, bkbytes, S, nS, wS, pkoff, pkbytes, proj, nproj, out, out_cap,
			sum_col, threads, res, 0);
}

int or_mergejoin_digest(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_col* proj, int nproj, int threads, or_digest* dg)
{
	or_join_result res;
	memset(dg, 0, sizeof *dg);
	return mergejoin_run(R, nR, wR, bkoff, bkbytes, S, nS, wS, pkoff, pkbytes, proj, nproj, 0, 0, -1,
			threads, &res, dg);
}

static int mergejoin_run(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_col* proj, int nproj, void* out, uint64_t out_cap,
		int sum_col, int threads, or_join_result* res, or_digest* dg)
{
	if (threads < 1) threads = 1;
	uint32_t ow = 0;
	for (int j = 0; j < nproj; ++j) ow += proj[j].bytes;
	if (ow > 1024) return -1;
	pthread_barrier_t bar; pthread_barrier_init(&bar, 0, threads);
	kidx** rruns = (kidx**) calloc(threads, sizeof(kidx*));
	kidx** sruns = (kidx**) calloc(threads, sizeof(kidx*));
	uint64_t* lens = (uint64_t*) calloc(4 * threads, sizeof(uint64_t));
	mj_arg* args = (mj_arg*) calloc(threads, sizeof(mj_arg));
	for (int t = 0; t < threads; ++t) {
		mj_arg* a = &args[t];
		a->R = (const char*) R; a->S = (const char*) S; a->nR = nR; a->nS = nS;
		a->wR = wR; a->wS = wS; a->bkoff = bkoff; a->bkbytes = bkbytes;
		a->pkoff = pkoff; a->pkbytes = pkbytes; a->proj = proj; a->nproj = nproj;
		a->ow = ow; a->sum_col = sum_col; a->T = threads; a->tid = t; a->materialise = out != 0;
		a->digest = dg != 0;
		a->rruns = rruns; a->sruns = sruns; a->rlen = lens; a->slen = lens + threads;
		a->rlo = lens + 2 * threads; a->slo = lens + 3 * threads; a->bar = &bar;
	}
	run_threads(threads, mj_thread, args, sizeof(mj_arg));
	uint64_t total = 0, written = 0; int64_t sum = 0;
	for (int t = 0; t < threads; ++t) {
		mj_arg* a = &args[t];
		total += a->nout; sum = (int64_t) ((uint64_t) sum + (uint64_t) a->sum);
		if (dg) dg_merge(dg, &a->dg);
		if (out) {
			uint64_t rows = a->out.used / ow, take = rows;
			if (written + take > out_cap) take = out_cap > written ? out_cap - written : 0;
			memcpy((char*) out + written * ow, a->out.data, take * ow);
			written += take;
		}
		free(a->out.data); free(rruns[t]); free(sruns[t]);
	}
	free(args); free(rruns); free(sruns); free(lens); pthread_barrier_destroy(&bar);
	res->n_out = total; res->sum = sum;
	return 0;
}

/* ------------------------------------------------------------------ */
/* Filter and Project: filter.cpp:37-85, project.cpp:37-104            */
/* ------------------------------------------------------------------ */

/* The raw comparison functions of rawcompfns.cpp for equal types: the left
 * operand is the column, the right one Filter's parsed constant
 * (Comparator::eval, comparator.h:72-76). */
static int or_cmp_sign_ok(uint32_t op, int lt, int eq, int gt)
{
	switch (op) {
	case OR_CMP_EQ: return eq;
	case OR_CMP_NE: return !eq;
	case OR_CMP_LT: return lt;
	case OR_CMP_LE: return lt || eq;
	case OR_CMP_GT: return gt;
	default: return gt || eq;
	}
}

static int or_pred_one(const or_pred* p, const char* t)
{
	const char* c = t + p->off;
	if (p->type == OR_PRED_INT) {
		int32_t a, b;
		memcpy(&a, c, 4); memcpy(&b, p->value, 4);
		return or_cmp_sign_ok(p->op, a < b, a == b, a > b);
	}
	if (p->type == OR_PRED_LONG) {
		int64_t a, b;
		memcpy(&a, c, 8); memcpy(&b, p->value, 8);
		return or_cmp_sign_ok(p->op, a < b, a == b, a > b);
	}
	if (p->type == OR_PRED_DEC) {
		/* DoubleDouble* (rawcompfns.cpp:294-327): C comparisons, so a NaN
		 * is unequal to everything and only != holds. */
		double a, b;
		memcpy(&a, c, 8); memcpy(&b, p->value, 8);
		switch (p->op) {
		case OR_CMP_EQ: return a == b;
		case OR_CMP_NE: return a != b;
		case OR_CMP_LT: return a < b;
		case OR_CMP_LE: return a <= b;
		case OR_CMP_GT: return a > b;
		default: return a >= b;
		}
	}
	/* CharChar* (rawcompfns.cpp:329-357): strncmp over the column width
	 * (Comparator::init, comparator.cpp:368). */
	int d = strncmp(c, (const char*) p->value, p->bytes);
	return or_cmp_sign_ok(p->op, d < 0, d == 0, d > 0);
}

/* Filter::map over every tuple (filter.cpp:76-85): a tuple is copied out
 * when the comparator holds; Filter over Filter is the conjunction. */
uint64_t or_filter(const void* in, uint64_t n, uint32_t w, const or_pred* preds, int npred, void* out)
{
	const char* src = (const char*) in;
	char* dst = (char*) out;
	uint64_t m = 0;
	for (uint64_t i = 0; i < n; ++i) {
		const char* t = src + i * w;
		int ok = 1;
		for (int k = 0; k < npred && ok; ++k) ok = or_pred_one(&preds[k], t);
		if (ok) { memcpy(dst + m * w, t, w); ++m; }
	}
	return m;
}

/* Project::map (project.cpp:93-104): the listed columns written in order. */
void or_project(const void* in, uint64_t n, uint32_t w, const or_col* cols, int ncols, void* out)
{
	const char* src = (const char*) in;
	char* dst = (char*) out;
	for (uint64_t i = 0; i < n; ++i)
		for (int c = 0; c < ncols; ++c) {
			memcpy(dst, src + i * w + cols[c].off, cols[c].bytes);
			dst += cols[c].bytes;
		}
}
