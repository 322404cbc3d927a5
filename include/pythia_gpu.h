/*
 * pythia_gpu.h — C ABI of the GB300 (sm_103a) execution path for Pythia's
 * data-parallel operators: radix/range partitioning, hash-join build and
 * probe, group-by aggregate_sum / aggregate_count, the page sort and the
 * MPSM sort-merge join.
 *
 * Plain C: pointers, sizes and status codes only; nothing here throws.
 * Relations are arrays of fixed-width row-major tuples exactly as Pythia's
 * Page/TupleBuffer holds them (util/buffer.h:134-337) with the column layout
 * of Schema (schema.h:148-350: packed, offsets = running sum of widths;
 * int 4 B, long/dec/date 8 B). All data pointers are DEVICE pointers unless a
 * function's name ends in _host. A `stream` is a cudaStream_t (NULL = the
 * legacy default stream).
 *
 * Each entry point names the reference interface it replaces.
 */
#ifndef PYTHIA_GPU_H
#define PYTHIA_GPU_H
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes (Operator::ResultCode Error, operators/operators.h:89-93,
 *      is the caller's mapping of every non-zero value) ---- */
#define PG_OK               0
#define PG_ERR_ARG          1  /* invalid argument or unsupported layout          */
#define PG_ERR_OOM          2  /* device allocation failed                        */
#define PG_ERR_CUDA         3  /* a CUDA runtime call failed                      */
#define PG_ERR_TIMEOUT      4  /* a bounded device-side wait gave up               */
#define PG_ERR_TABLE_FULL   5  /* hash table probe sequence exhausted             */
#define PG_ERR_OUTPUT_FULL  6  /* output capacity too small; *n_out = rows needed */
#define PG_ERR_UNSUPPORTED  7  /* configuration the library does not implement    */

typedef struct pg_ctx pg_ctx;
typedef struct pg_hashtable pg_hashtable;
typedef void* pg_stream;

/* ---- hash function descriptor: the plan's `hash` node as
 *      TupleHasher::create reads it (hash.cpp:99-234) ---- */
enum {
	PG_FN_BYTES = 0, PG_FN_MODULO = 1, PG_FN_RANGE = 2, PG_FN_EXACTRANGE = 3,
	PG_FN_PARAMMODULO = 4, PG_FN_KNUTH = 5, PG_FN_TPCHORDERKEY = 6,
	PG_FN_WILLIS = 7, PG_FN_ALWAYSZERO = 8, PG_FN_TPCHQ1MAGIC = 9
};
typedef struct {
	int32_t fn;          /* PG_FN_*                                   */
	uint32_t buckets;    /* "buckets"                                 */
	int64_t min, max;    /* "range" = [min, max] (range, exactrange)  */
	uint32_t skipbits;   /* "skipbits" (parammodulo, knuth)           */
	uint32_t offset;     /* "offset"   (parammodulo)                  */
} pg_hashcfg;

/* A relation: n tuples of `width` bytes; the key column at key_off,
 * key_bytes = 4 (int) or 8 (long/date), or 0 where no key applies. */
typedef struct {
	const void* data;
	uint64_t n;
	uint32_t width;
	uint32_t key_off;
	uint32_t key_bytes;
} pg_rel;

/* One output column of a join projection ("B$i" / "P$i",
 * createProjectionVector, operators/join.cpp:141-182): side 0 = build,
 * 1 = probe; byte offset and width of the column in that side's tuple. */
typedef struct {
	uint32_t side;
	uint32_t off;
	uint32_t bytes;
} pg_col;

/* Join outcome. n_out counts output rows whether or not they were written. */
typedef struct {
	uint64_t n_out;
	int64_t sum;        /* wrapping int64 sum of output column sum_col  */
} pg_join_result;

enum { PG_JOIN_MATERIALIZE = 1, PG_JOIN_COUNT = 2, PG_JOIN_SUM = 4 };
/* pg_mpsm_join only: that side is already sorted on its key, as a plan's
 * buildpresorted / probepresorted = "yes" states (SortMergeJoinOp::init,
 * operators/join.cpp:750-762). The device confirms it while it reads the key
 * range and then skips that side's sort or partition; a side that is not
 * sorted is sorted as usual, so the result never depends on the flags. */
enum { PG_JOIN_BUILD_SORTED = 8, PG_JOIN_PROBE_SORTED = 16 };

/* ---------------------------------------------------------------------- */
/* Context, memory, streams (replace numaallocate_*, util/numaallocate.h:35-37,
 * and the per-operator thread/barrier plumbing of MergeOp)                */
/* ---------------------------------------------------------------------- */
int pg_init(int device, uint64_t reserved_bytes, pg_ctx** ctx);
int pg_shutdown(pg_ctx* ctx);
const char* pg_last_error(pg_ctx* ctx);
int pg_device_status(pg_ctx* ctx);             /* sticky device error word  */
int pg_stream_create(pg_ctx* ctx, pg_stream* stream);
/* A stream whose kernels the block scheduler prefers to those of ordinary
 * streams (highest CUDA stream priority): short requests run ahead of long
 * ones sharing the GPU. */
int pg_stream_create_urgent(pg_ctx* ctx, pg_stream* stream);
int pg_stream_destroy(pg_ctx* ctx, pg_stream stream);
int pg_sync(pg_ctx* ctx, pg_stream stream);
int pg_buffer_alloc(pg_ctx* ctx, uint64_t bytes, void** dptr);
int pg_buffer_free(pg_ctx* ctx, void* dptr);
/* Stream-ordered device buffers from the context's pool: no device-wide
 * synchronisation, so queries on other streams keep running. */
int pg_buffer_alloc_async(pg_ctx* ctx, pg_stream stream, uint64_t bytes, void** dptr);
int pg_buffer_free_async(pg_ctx* ctx, pg_stream stream, void* dptr);
int pg_host_alloc(pg_ctx* ctx, uint64_t bytes, void** hptr);   /* pinned */
int pg_host_free(pg_ctx* ctx, void* hptr);
/* Page-locks existing host memory (a relation a loader read into memory) so
 * that copies from it run at the host link's rate; pg_host_is_pinned tells
 * whether a host pointer lies in pinned or registered memory (1) or not (0). */
int pg_host_register(pg_ctx* ctx, void* hptr, uint64_t bytes);
int pg_host_unregister(pg_ctx* ctx, void* hptr);
int pg_host_is_pinned(pg_ctx* ctx, const void* hptr);
/* 1 when this context's kernels can read host pointer hptr directly: pinned
 * or registered memory, or any host memory on a device that reads pageable
 * memory (cudaDevAttrPageableMemoryAccess, e.g. over NVLink-C2C); else 0. */
int pg_host_readable(pg_ctx* ctx, const void* hptr);
/* Host-to-device copy made by the SMs' loads of host memory instead of a
 * copy engine; src must be readable (pg_host_readable), any alignment, and
 * stay mapped until the copy has run: unlike pg_h2d, which reports a bad host
 * range as an error, the kernel's loads of an unmapped address fault it.
 * Replaces the page hand-over of ParallelScanOp (operators/parallelscan.cpp:
 * 176-190) for pages a GPU operator uploads one at a time: measured 181 GB/s
 * for 1 MB pages from 16 threads, against 117 GB/s by copy engine. */
int pg_h2d_sm(pg_ctx* ctx, pg_stream stream, void* dst, const void* src, uint64_t bytes);
int pg_h2d(pg_ctx* ctx, pg_stream stream, void* dst, const void* src, uint64_t bytes);
int pg_d2h(pg_ctx* ctx, pg_stream stream, void* dst, const void* src, uint64_t bytes);
int pg_d2d(pg_ctx* ctx, pg_stream stream, void* dst, const void* src, uint64_t bytes);
int pg_memset(pg_ctx* ctx, pg_stream stream, void* dst, int value, uint64_t bytes);
/* Number of kernels this library has launched (process-wide). */
uint64_t pg_kernel_launches(void);

/* Launch-shape knobs of a context, set by the autotuner (pythia_gb300/autotune.py).
 * No reference counterpart: they replace the reference's compile-time and plan
 * constants that size per-thread work (buffsize, tuplesperbucket, thread counts).
 * Value 0 restores the built-in choice. Results never depend on them; a low
 * PG_TUNE_SPIN_LIMIT can make a call fail with PG_ERR_TIMEOUT, which is how the
 * bounded device waits are tested. */
enum {
	PG_TUNE_PROBE_CTAS_PER_SM = 0,   /* resident 8-warp CTAs per SM of the 16-byte probe (1..5) */
	PG_TUNE_PROBE_VARIANT = 1,       /* 16-byte probe: 0 default, 1 warp-staged (bulk copies), 2 tiled with
	                                    bulk stores, 3 register loads with one-chunk prefetch (dense default
	                                    for other projections), 4 register loads without prefetch, 5 deeper
	                                    pipeline (default for (P$1, B$1) rows of narrow dense tables) */
	PG_TUNE_DENSE = 2,               /* 1: allow dense tables (default), 2: always hash */
	PG_TUNE_PARTITION_TILE = 3,      /* partition tile bytes (8192..65536) */
	PG_TUNE_GROUPBY_SMEM_GROUPS = 4, /* largest group count aggregated in shared memory first */
	PG_TUNE_RADIX_BITS = 5,          /* radix sort digit: 4..12 bits (partition fan-out 2^bits) */
	PG_TUNE_PROBE_ITEMS = 6,         /* dense-table lookups in flight per lane of the 16-byte probe: 4 or 8 */
	PG_TUNE_PROBE_CACHE = 7,         /* 16-byte probe L2 policies: bits 0-1 table loads (0 evict-last,
	                                    1 normal, 2 unchanged, 3 first), bit 2 probe reads and bit 3
	                                    output stores normal instead of evict-first, bits 4-6 evict-last
	                                    for that many eighths of the table's lines only (0: all), bit 7
	                                    table loads kept in L1 (dense-table probes); 0 = the built-in
	                                    4/8 evict-last with L1 (bits 4-7 = 0xC), 256 = all bits clear */
	PG_TUNE_PROBE_PASSES = 8,        /* dense-table probe passes: 1, 2 (half the table each), 0 by size */
	PG_TUNE_GROUPBY_PATH = 9,        /* group-by: 0 by key range and size, 1 hashed global table, 2 partitioned,
	                                    3 hashed global without warp combining, 4 partitioned without warp
	                                    combining, 6 dense when the key range allows, 7 as 6 without the
	                                    shared-memory tables of windows up to 4096 keys */
	PG_TUNE_PROBE_WIDE = 10,         /* probe of tuples or rows other than 16 bytes: 0 materialised rows of dense
	                                    tables staged through shared memory where the width allows, everything
	                                    else per-thread loads; 1 per-thread loads; 2 staged, 4 lookups per
	                                    thread; 3 staged, 2 lookups per thread */
	PG_TUNE_BUILD_SPEC = 11,         /* narrow dense build of 16-byte tuples: 0 on the device alone (key window
	                                    from a sample, checked by the table's first use) for 65,536 tuples or
	                                    more, 1 on the device alone at every size, 2 exact key range read back
	                                    to the host first */
	PG_TUNE_SPIN_LIMIT = 12,         /* polls a device-side wait for a bulk copy makes before the call fails with
	                                    PG_ERR_TIMEOUT (the copy is still waited for, so the kernel ends
	                                    cleanly): 0 the built-in limit (2^26 blocking polls), else that many
	                                    non-blocking polls */
	PG_TUNE_L2_FETCH = 13,           /* L2 fetch granularity hint of the context in bytes: 0 leaves the CUDA
	                                    default, else 32, 64 or 128 (cudaLimitMaxL2FetchGranularity, a limit of
	                                    the calling process that ends with it) */
	PG_TUNE_SORT_PATH = 14,          /* page sort and the MPSM's sorts: 0 LSD radix over key - min while the span
	                                    fits 63 bits (bitonic tiles and merge-path merges for wider spans and for
	                                    inputs of at most 2^18 tuples whose span needs over 32 bits), 1 radix
	                                    whenever the span fits 63 bits, 2 bitonic tiles and merges always */
	PG_TUNE_GROUPBY_ILP = 15,        /* rows in flight per thread of the dense group-by over a global table: 4
	                                    or 8 (0: built-in, 4 for dec sums, 8 otherwise) */
	PG_TUNE_HASH_PARTITION = 16,     /* hashed tables: 2 partitions the probe side (and R, for packed values) on
	                                    the keys' hash first, so that each partition uses a 16 MB slice of the
	                                    table; 0 (built-in) or 1: not (measured slower on the 16M x 256M
	                                    sparse-key join) */
	PG_TUNE_COUNT = 17
};
int pg_tune_set(pg_ctx* ctx, int knob, int64_t value);
int64_t pg_tune_get(pg_ctx* ctx, int knob);

/* ---------------------------------------------------------------------- */
/* Tuple hashing: TupleHasher::hash over a column (hash.h:85-124) with the
 * bucket functions of hash.h:150-479. out[i] = bucket of tuple i.        */
/* ---------------------------------------------------------------------- */
int pg_hash_buckets(pg_ctx* ctx, const pg_hashcfg* cfg, uint32_t* nbuckets);
int pg_hash_tuples(pg_ctx* ctx, pg_stream stream, const pg_rel* in,
		const pg_hashcfg* cfg, uint32_t* out);

/* ---------------------------------------------------------------------- */
/* Partition: PartitionOp::scanStart histogram / prefix / scatter
 * (operators/partition.cpp:166-359). Stable: within a partition tuples keep
 * input order, as the reference's per-thread prefix sums make them when
 * threads read consecutive slices. offsets (device, nbuckets+1 uint64)
 * receive partition starts, offsets[nbuckets] = n. Any hash function with
 * at most 4096 buckets; every tuple must hash below buckets().          */
/* ---------------------------------------------------------------------- */
int pg_partition(pg_ctx* ctx, pg_stream stream, const pg_rel* in,
		const pg_hashcfg* cfg, void* out, uint64_t* offsets);

/* Optional per-partition sort ("sort" = "yes", partition.cpp:83-95, 339-353):
 * sorts each partition of `data` in place by its key column. */
int pg_partition_sort(pg_ctx* ctx, pg_stream stream, const pg_rel* data,
		const uint64_t* offsets_host, uint32_t nbuckets, void* scratch_out);

/* ---------------------------------------------------------------------- */
/* Hash join build/probe: HashJoinOp::buildFromPage + scanStart (build,
 * operators/join.cpp:396-464, 641-667) and HashJoinOp::getNext
 * (probe, join.cpp:503-562) with constructOutputTuple (join.cpp:475-501).
 * Equi-join on R.key = S.key; duplicates on either side give every pair.
 * `proj` lists the output columns in order. Output rows are packed to the
 * sum of the projected widths; their order is unspecified.
 * pg_hashjoin_build may return while its kernels still read R, and the
 * table's first use may rebuild it from R (a dense layout taken from a
 * sample and then refuted): R must stay valid and unchanged until the
 * first probe (or other use) of the table has returned.                  */
/* ---------------------------------------------------------------------- */
int pg_hashjoin_build(pg_ctx* ctx, pg_stream stream, const pg_rel* R,
		const pg_col* proj, int nproj, pg_hashtable** ht);
int pg_hashjoin_probe(pg_ctx* ctx, pg_stream stream, pg_hashtable* ht,
		const pg_rel* S, const pg_col* proj, int nproj,
		void* out, uint64_t out_capacity, int flags, int sum_col,
		pg_join_result* res);
int pg_hashtable_free(pg_ctx* ctx, pg_hashtable* ht);

/* Table images: HashTable::serialize / deserialize (util/hashtable.cpp:99-201)
 * with the segment files of creatememsegment (operators/memsegmentwriter.cpp:
 * 154-197) and attachmemsegment (util/hashtable.cpp:124-178). An image is a
 * 512-byte self-describing header (layout, key domain, build projection,
 * checksums) and the table's arrays; loading needs no build relation and no
 * table parameters. Tables that store build row indices (build-projected
 * columns wider than 8 bytes) are not self-contained: PG_ERR_UNSUPPORTED.
 *
 * pg_hashtable_image_size: bytes of the image of `ht`.
 * pg_hashtable_serialize: writes the image into host memory `image`
 *   (pinned memory from pg_host_alloc copies fastest); *bytes = image size.
 *   image == NULL only reports the size; a smaller capacity gives
 *   PG_ERR_OUTPUT_FULL.
 * pg_hashtable_deserialize: a new table on this context's device from an
 *   image in host memory; a damaged image (magic, version, layout, sizes,
 *   header or payload checksum) gives PG_ERR_ARG and no table. The table is
 *   probed, grouped and freed like one from pg_hashjoin_build.
 * pg_hashtable_save / _load: the same through a file; save creates a new
 *   file and fails if `path` exists, as the reference's segment writer does. */
int pg_hashtable_image_size(pg_ctx* ctx, const pg_hashtable* ht, uint64_t* bytes);
int pg_hashtable_serialize(pg_ctx* ctx, pg_stream stream, const pg_hashtable* ht,
		void* image, uint64_t capacity, uint64_t* bytes);
int pg_hashtable_deserialize(pg_ctx* ctx, pg_stream stream, const void* image, uint64_t bytes,
		pg_hashtable** ht);
int pg_hashtable_save(pg_ctx* ctx, pg_stream stream, const pg_hashtable* ht, const char* path);
int pg_hashtable_load(pg_ctx* ctx, pg_stream stream, const char* path, pg_hashtable** ht);

/* Whole operator through HOST buffers (the call a Page-draining operator
 * makes): copies in, builds, probes, copies out. Chunked so copies overlap
 * the probe. out_host may be NULL with flags lacking PG_JOIN_MATERIALIZE. */
int pg_hashjoin_host(pg_ctx* ctx, const pg_rel* R_host, const pg_rel* S_host,
		const pg_col* proj, int nproj, void* out_host, uint64_t out_capacity,
		int flags, int sum_col, pg_join_result* res);

/* Join count/sum that allocates nothing. No counterpart in the reference: an
 * addition for callers that may not allocate device memory while a query runs
 * (a host that owns the device's memory through its own pool, a sandbox with a
 * fixed budget, a latency-critical path that must not reach the allocator).
 * Computes pg_hashjoin_build + pg_hashjoin_probe(PG_JOIN_COUNT | PG_JOIN_SUM):
 * res->n_out = join rows, res->sum = wrapping sum of output column sum_col
 * (-1: none). The hash table lives in one fixed 16 MiB device array that the
 * library declares; the build side may hold at most 524288 tuples (PG_ERR_ARG
 * beyond), and build-side projected columns at most 8 bytes in total. The
 * first call on each device in a process loads the library's device code and
 * places the array there (CUDA loads modules lazily), which can allocate
 * device memory: make it, with empty inputs if need be, before a pool takes
 * the device's memory; later calls allocate nothing. Runs on ctx's device
 * whatever device is current. Synchronous (returns after the result is on
 * the host), so never call it while a stream is being captured. Calls share
 * the array (each clears it first), so calls that overlap on the GPU race. */
int pg_hashjoin_agg_noalloc(pg_ctx* ctx, pg_stream stream, const pg_rel* R,
		const pg_rel* S, const pg_col* proj, int nproj, int sum_col,
		pg_join_result* res);

/* ---------------------------------------------------------------------- */
/* Filter and Project: Filter::map and Project::map (operators/filter.cpp:
 * 37-85, project.cpp:37-104) over MapWrapper's per-thread page loop
 * (mapwrapper.cpp:38-138), one launch per relation. A predicate compares one
 * column with a constant of the column's own type, as Filter's Comparator
 * does (comparator.cpp:43-433, rawcompfns.cpp): int, long and date as signed
 * integers, dec as double (IEEE: NaN compares unequal), char as strncmp over
 * the column width. Several predicates form a conjunction (a Filter over a
 * Filter).                                                                 */
/* ---------------------------------------------------------------------- */
enum { PG_PRED_INT = 1, PG_PRED_LONG = 2, PG_PRED_DEC = 3, PG_PRED_CHAR = 4 };
enum { PG_CMP_EQ = 0, PG_CMP_NE = 1, PG_CMP_LT = 2, PG_CMP_LE = 3, PG_CMP_GT = 4, PG_CMP_GE = 5 };
#define PG_PRED_MAX 4
typedef struct {
	uint32_t type;          /* PG_PRED_* (a date column: PG_PRED_LONG)            */
	uint32_t op;            /* PG_CMP_*: column <op> value                         */
	uint32_t off;           /* byte offset of the column, a multiple of 4 (char: any) */
	uint32_t bytes;         /* 4 (int), 8 (long, dec), 1..128 (char)               */
	uint8_t value[128];     /* the constant as the column stores it (char: strncpy'd) */
} pg_pred;
/* Stable: out = the tuples of `in` satisfying every predicate, in input
 * order; *n_out = their number. `out` has room for in->n tuples.          */
int pg_filter(pg_ctx* ctx, pg_stream stream, const pg_rel* in, const pg_pred* preds, int npred,
		void* out, uint64_t* n_out);
/* out[i] = the columns cols[0..ncols) of in[i] (byte offset `off`, width
 * `bytes`, multiples of 4; `side` ignored), packed in order.               */
int pg_project(pg_ctx* ctx, pg_stream stream, const pg_rel* in, const pg_col* cols, int ncols, void* out);
/* pg_hashjoin_probe over the probe tuples that satisfy `preds`: the Filter
 * under a join's probe side run as the probe's prologue. For 16-byte probe
 * tuples of a dense table and predicates on int/long/dec columns the probe
 * kernel evaluates them before its table lookups (no filtered copy of S);
 * otherwise S is filtered first.                                          */
/* pg_hashjoin_probe over a probe side held as `nspans` separate arrays (the
 * pages several engine threads uploaded), as if they were one relation:
 * same rows (order across spans unspecified), count and sum, without first
 * copying the spans together. All spans share width and key position.
 * Tables with repeated build keys: PG_ERR_UNSUPPORTED (gather and use
 * pg_hashjoin_probe). Replaces HashJoinOp's probe of each thread's own pages
 * against its group's table (getNext and readNextTupleFromProbe,
 * operators/join.cpp:503-603). */
int pg_hashjoin_probe_spans(pg_ctx* ctx, pg_stream stream, pg_hashtable* ht, const pg_rel* spans, int nspans,
		const pg_col* proj, int nproj, void* out, uint64_t out_capacity, int flags, int sum_col,
		pg_join_result* res);
int pg_hashjoin_probe_where(pg_ctx* ctx, pg_stream stream, pg_hashtable* ht, const pg_rel* S,
		const pg_pred* preds, int npred, const pg_col* proj, int nproj,
		void* out, uint64_t out_capacity, int flags, int sum_col, pg_join_result* res);

/* ---------------------------------------------------------------------- */
/* Group-by: GenericAggregate::remember + AggregateSum / AggregateCount fold
 * (operators/genericaggregate.cpp:240-487, aggregatesum.cpp:53-107,
 * aggregatecount.cpp:37-52). Key: in->key_bytes 4 or 8, or 0 for no GROUP BY
 * (the "alwayszero" plan). Output rows: (key, agg) packed; agg is int32 for
 * an int sum (wrapping, as the reference's CtInt +=), int64 for a long sum or
 * a count, double for a dec sum. Integer results are exact; dec sums are exact
 * fixed-point sums rounded once (the correctly rounded sum whenever the values
 * lie within 2^133 of the column's largest; the same bits in any row order);
 * infinities and NaNs give IEEE's result for their groups.
 * groups_hint sizes the table (0: n).                                      */
/* ---------------------------------------------------------------------- */
enum { PG_VAL_INT = 0, PG_VAL_LONG = 1, PG_VAL_DEC = 2 };
enum { PG_AGG_SUM = 0, PG_AGG_COUNT = 1 };
int pg_groupby(pg_ctx* ctx, pg_stream stream, const pg_rel* in,
		uint32_t val_off, int val_type, int agg, uint64_t groups_hint,
		void* out, uint64_t out_capacity, uint64_t* ngroups);

/* Join then group-by without writing the join rows: a HashJoinOp whose output
 * feeds AggregateSum / AggregateCount grouped on the build-side column
 * (join.cpp:503-562 + genericaggregate.cpp:240-282). `ht` must have been built
 * with exactly one build-side projected column (the group key, 4 or 8 bytes);
 * the probe column at val_off (val_type) is summed, or matches are counted.
 * Output rows as pg_groupby: (group, agg), order unspecified; dec sums exact
 * as pg_groupby's. Needs a narrow dense table whose group values span a
 * compact range and 16-byte probe tuples, and a summed dec column free of
 * infinities and NaNs; otherwise PG_ERR_UNSUPPORTED, and the caller probes
 * (materialised) and groups in two steps.                                 */
int pg_hashjoin_groupby(pg_ctx* ctx, pg_stream stream, pg_hashtable* ht, const pg_rel* S,
		uint32_t val_off, int val_type, int agg, void* out, uint64_t out_capacity, uint64_t* ngroups);

/* ---------------------------------------------------------------------- */
/* Page sort: TupleBuffer::sort<KeyT> / sortAllInPage (util/buffer.inl:135-292,
 * operators/join.cpp:893-912) and the bitonic block sort
 * (util/bitonicsort.cpp:371-443): bitonic sort of `tile`-tuple pages in
 * shared memory, then merge-path merges. Ascending signed key; ties in
 * unspecified order. `out` may not alias `in`.                            */
/* ---------------------------------------------------------------------- */
int pg_sort_pages(pg_ctx* ctx, pg_stream stream, const pg_rel* in, void* out);

/* ---------------------------------------------------------------------- */
/* MPSM / sort-merge join: SortMergeJoinOp::BufferAndSort + OldMPSMJoinOp /
 * MPSMJoinOp merge (operators/join.cpp:945-1371, 1383-1538). Same output
 * contract as pg_hashjoin_probe.                                          */
/* ---------------------------------------------------------------------- */
int pg_mpsm_join(pg_ctx* ctx, pg_stream stream, const pg_rel* R, const pg_rel* S,
		const pg_col* proj, int nproj, void* out, uint64_t out_capacity,
		int flags, int sum_col, pg_join_result* res);

/* ---------------------------------------------------------------------- */
/* Batched uneven joins: many independent join + aggregate_count instances
 * (one HashJoinOp plan per instance under MergeOp in the reference,
 * operators/join.cpp:273-675, aggregatecount.cpp:37-52) run by one build and
 * one probe launch over instance-aligned tiles, optionally replayed as a CUDA
 * graph. Relations are 16-byte (long key, long payload) tuples keyed at 0;
 * counts[i] = number of join rows of instance i.                          */
/* ---------------------------------------------------------------------- */
typedef struct {
	const void* R; uint64_t nR;      /* build relation (device)  */
	const void* S; uint64_t nS;      /* probe relation (device)  */
} pg_batch_item;
typedef struct {
	int32_t threads;       /* 128, 256 or 512 threads per CTA                */
	int32_t items;         /* probe keys in flight per thread: 1, 2, 4, 8    */
	uint32_t tile;         /* tuples per tile                                */
	int32_t ctas_per_sm;   /* persistent CTAs per SM                         */
	int32_t load_inverse;  /* table slots per build tuple (2: load 1/2)      */
	int32_t use_graph;     /* capture clear+build+probe as a CUDA graph      */
} pg_batch_shape;
typedef struct pg_batch pg_batch;
int pg_batch_prepare(pg_ctx* ctx, pg_stream stream, const pg_batch_item* items, uint32_t n,
		const pg_batch_shape* shape, pg_batch** batch);
int pg_batch_run(pg_ctx* ctx, pg_batch* batch, uint64_t* counts_host);
int pg_batch_free(pg_ctx* ctx, pg_batch* batch);
/* Launch-shape autotuner over batches (no reference counterpart: the reference
 * has no tunables at this level): prepares, warms and times each of the
 * n_shapes candidate shapes on these instances (CUDA events, best of
 * `repeats`), returns the fastest index in *best and each shape's time in
 * ms_out[] (n_shapes entries, may be NULL). */
int pg_autotune_batch(pg_ctx* ctx, pg_stream stream, const pg_batch_item* items, uint32_t n,
		const pg_batch_shape* shapes, uint32_t n_shapes, int repeats, uint32_t* best, double* ms_out);
/* Synthetic foreign keys for benchmarks: S[j] = (R[h(seed, j) mod nR].key,
 * h'(seed, j)), 16-byte tuples, h a SplitMix64 counter hash. */
int pg_generate_fk(pg_ctx* ctx, pg_stream stream, const void* R, uint64_t nR, uint64_t seed,
		void* S, uint64_t nS);
/* As pg_generate_fk with Zipf(s) ranks over R's rows (rejection-inversion,
 * Hormann-Derflinger 1996; s = 0 is uniform) and a dec payload uniform in
 * [0, vmax): S[j] = (R[rank - 1].key, value). */
int pg_generate_zipf_fk(pg_ctx* ctx, pg_stream stream, const void* R, uint64_t nR, double s,
		uint64_t seed, void* S, uint64_t nS, double vmax);

#ifdef __cplusplus
}
#endif
#endif
