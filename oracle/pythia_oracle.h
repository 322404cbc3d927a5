/*
 * TEST INFRASTRUCTURE — the oracle. Not part of the product.
 *
 * A plain-C restatement of the reference Pythia CPU operators on the GPU
 * path: the tuple hash functions, the chained-bucket hash join, the stable
 * exactrange/radix partition, the hash aggregates, the page sort and the
 * sort-merge (MPSM) join. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference arm call it, always as the checker or the timed
 * CPU baseline, never as the thing measured or shipped.
 *
 * Every function cites the reference file:line it restates. Parity of this
 * restatement is pinned against the reference itself (the engine compiled
 * from its own sources by oracle/Makefile.ref, outputs committed under
 * tests/golden/) and the reference unit tests' known answers.
 */
#ifndef PYTHIA_ORACLE_H
#define PYTHIA_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Hash function kinds accepted by TupleHasher::create (hash.cpp:99-234). */
enum {
	OR_FN_BYTES = 0, OR_FN_MODULO = 1, OR_FN_RANGE = 2, OR_FN_EXACTRANGE = 3,
	OR_FN_PARAMMODULO = 4, OR_FN_KNUTH = 5, OR_FN_TPCHORDERKEY = 6,
	OR_FN_WILLIS = 7, OR_FN_ALWAYSZERO = 8, OR_FN_TPCHQ1MAGIC = 9
};

/* Configuration as read from a plan's hash node, before derivation. */
typedef struct {
	int32_t fn;
	uint32_t buckets;   /* "buckets" */
	int64_t min, max;   /* "range" = (min, max) */
	uint32_t skipbits;  /* "skipbits" */
	uint32_t offset;    /* "offset" (read as unsigned int, hash.cpp:182-185) */
} or_hashcfg;

/* Derived state, as the HashFunction constructors leave it. */
typedef struct {
	int32_t fn;
	int64_t k;          /* HashFunction::_k, with each subclass's reuse of it */
	int64_t min, max;
	int64_t bucketrange;
	uint32_t skipbits;
	uint32_t nbuckets;  /* buckets() */
} or_hashfn;

uint32_t or_getlogarithm(uint32_t k);
int or_hashfn_make(const or_hashcfg* cfg, or_hashfn* out);
uint32_t or_hash_value(const or_hashfn* f, const void* field, uint32_t size);
void or_hash_column(const or_hashfn* f, const void* rows, uint64_t n, uint32_t w,
		uint32_t off, uint32_t size, uint32_t* out);
int64_t or_exactrange_minimumforbucket(const or_hashfn* f, uint32_t bucket);
/* ParameterizedModuloValueHasher::generate: writes `passes` derived configs. */
int or_parammodulo_generate(const or_hashfn* f, uint32_t passes, or_hashfn* out);

/* Projection column: side 0 = build ("B$i"), 1 = probe ("P$i"). */
typedef struct { uint32_t side, off, bytes; } or_col;

typedef struct {
	uint64_t n_out;      /* rows produced (even when out is NULL or full) */
	int64_t sum;         /* wrapping int64 sum of output column sum_col */
} or_join_result;

int or_hashjoin(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_hashcfg* hash, uint32_t tuplesperbucket,
		const or_col* proj, int nproj, void* out, uint64_t out_cap,
		int sum_col, int threads, or_join_result* res);

/* or_hashjoin with every output row written into one output page of
 * page_bytes per thread that is reused once full, as HashJoinOp::getNext
 * fills and hands on its output page (join.cpp:510-545): the CPU timing
 * of the reference operator, with no result array. */
int or_hashjoin_paged(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_hashcfg* hash, uint32_t tuplesperbucket,
		const or_col* proj, int nproj, uint32_t page_bytes,
		int sum_col, int threads, or_join_result* res);

/* Order-independent digest of a multiset of rows, all sums mod 2^64: the
 * row count, the sums of each row's first and second 8-byte words (zero
 * where a row is shorter) and the sum of a hash of each whole row. A
 * checker utility for outputs too large to compare row by row. */
typedef struct { uint64_t n, w0, w1, h; } or_digest;
void or_rows_digest(const void* rows, uint64_t n, uint32_t w, int threads, or_digest* d);
/* The digest of or_hashjoin's / or_mergejoin's output rows, without
 * materialising them. */
int or_hashjoin_digest(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_hashcfg* hash, uint32_t tuplesperbucket,
		const or_col* proj, int nproj, int threads, or_digest* d);

int or_partition(const void* in, uint64_t n, uint32_t w, uint32_t koff, uint32_t kbytes,
		const or_hashcfg* hash, void* out, uint64_t* offsets, int threads);

enum { OR_VAL_INT = 0, OR_VAL_LONG = 1, OR_VAL_DEC = 2 };
enum { OR_AGG_SUM = 0, OR_AGG_COUNT = 1 };
int or_groupby(const void* in, uint64_t n, uint32_t w, int has_key, uint32_t koff, uint32_t kbytes,
		uint32_t voff, int vtype, int agg, const or_hashcfg* hash,
		void* out, uint64_t out_cap, uint64_t* ngroups, int threads);
int or_groupby_exact(const void* in, uint64_t n, uint32_t w, int has_key, uint32_t koff,
		uint32_t kbytes, uint32_t voff, void* out, uint64_t out_cap, uint64_t* ngroups);
double or_fsum(const double* x, uint64_t n, uint64_t stride);

int or_sort(const void* in, uint64_t n, uint32_t w, uint32_t koff, uint32_t kbytes, void* out);

int or_mergejoin(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_col* proj, int nproj, void* out, uint64_t out_cap,
		int sum_col, int threads, or_join_result* res);
int or_mergejoin_digest(const void* R, uint64_t nR, uint32_t wR, uint32_t bkoff, uint32_t bkbytes,
		const void* S, uint64_t nS, uint32_t wS, uint32_t pkoff, uint32_t pkbytes,
		const or_col* proj, int nproj, int threads, or_digest* d);

/* Filter / Project (filter.cpp:37-85, project.cpp:37-104): column types and
 * comparisons of Comparator (comparator.h:43-83). A date column compares as
 * a long (CtDate is a long long, comparator.cpp:370-403). */
enum { OR_PRED_INT = 1, OR_PRED_LONG = 2, OR_PRED_DEC = 3, OR_PRED_CHAR = 4 };
enum { OR_CMP_EQ = 0, OR_CMP_NE = 1, OR_CMP_LT = 2, OR_CMP_LE = 3, OR_CMP_GT = 4, OR_CMP_GE = 5 };
typedef struct {
	uint32_t type, op, off, bytes;
	uint8_t value[128];
} or_pred;
/* Tuples satisfying every predicate, in input order; returns their number. */
uint64_t or_filter(const void* in, uint64_t n, uint32_t w, const or_pred* preds, int npred, void* out);
/* out[i] = columns (off, bytes) of in[i], packed in order. */
void or_project(const void* in, uint64_t n, uint32_t w, const or_col* cols, int ncols, void* out);

#ifdef __cplusplus
}
#endif
#endif
