// Internal definitions shared by the sm_103a kernels of libpythia_gpu.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <mutex>
#include <atomic>
#include "../../include/pythia_gpu.h"

// ---------------------------------------------------------------------------
// Context
// ---------------------------------------------------------------------------
struct pg_ctx {
	int device;
	int sm_count;
	int64_t tune[PG_TUNE_COUNT];   // launch-shape knobs, PG_TUNE_* (0 = built-in choice)
	cudaMemPool_t pool;
	cudaMemPool_t big_pool;  // allocations of PG_BIG_ALLOC bytes or more (NULL: all from `pool`)
	int* d_status;          // sticky device error word (PG_ERR_*), 0 = fine
	unsigned long long* d_scratch64;  // small per-context device scratch (counters)
	int pageable_access;    // kernels may read pageable host memory (cudaDevAttrPageableMemoryAccess)
	int host_ptr_registered;  // registered host memory is read through its host address
	std::mutex mu;
	std::string last_error;
};

extern std::atomic<uint64_t> g_kernel_launches;

int pg_fail(pg_ctx* ctx, int code, const std::string& msg);
int pg_cuda_fail(pg_ctx* ctx, cudaError_t e, const char* what);

#define PG_CUDA(ctx, call)                                                   \
	do {                                                                     \
		cudaError_t e_ = (call);                                             \
		if (e_ != cudaSuccess) return pg_cuda_fail((ctx), e_, #call);        \
	} while (0)

// Records a kernel launch and checks its configuration error.
#define PG_LAUNCHED(ctx)                                                     \
	do {                                                                     \
		g_kernel_launches.fetch_add(1, std::memory_order_relaxed);           \
		cudaError_t e_ = cudaGetLastError();                                 \
		if (e_ != cudaSuccess) return pg_cuda_fail((ctx), e_, "kernel launch"); \
	} while (0)

// Stream-ordered scratch from the context's pools (PG_BIG_ALLOC bytes and more
// from the large-buffer pool).
#define PG_BIG_ALLOC (256ull << 20)
int pg_alloc_async(pg_ctx* ctx, cudaStream_t s, void** p, size_t bytes);
void pg_free_async(pg_ctx* ctx, cudaStream_t s, void* p);
// Reads the sticky status after synchronising `s`; returns its PG_ERR_* code.
int pg_check_status(pg_ctx* ctx, cudaStream_t s, const char* what);
// Clears a non-zero status `st` read back by the caller and reports it.
int pg_status_fail(pg_ctx* ctx, cudaStream_t s, int st, const char* what);

// ---------------------------------------------------------------------------
// Bucket functions (hash.h:51-479) in the form their constructors leave them.
// ---------------------------------------------------------------------------
struct pg_hashfn {
	int32_t fn;
	int64_t k;            // HashFunction::_k as each subclass uses it
	int64_t min, max;
	int64_t bucketrange;
	uint32_t skipbits;
	uint32_t nbuckets;
};

int pg_hashfn_derive(const pg_hashcfg* c, pg_hashfn* f);
// Stable partition by a derived bucket function (pg_partition.cu); offsets may
// be null. Queues work on `s` without synchronising.
int pg_partition_fn(pg_ctx* ctx, cudaStream_t s, const pg_rel* in, const pg_hashfn& f,
		void* out, uint64_t* offsets);

// Internal bucket function (not a plan option): the top log2(buckets) bits of
// the 64-bit key mix, skipbits = 64 - log2(buckets). Spreads any key domain
// evenly, for partitions that feed per-partition tables.
#define PG_FN_MIXRADIX 64

__device__ __forceinline__ uint64_t pg_mix64(uint64_t k);

// Key columns are 4-byte aligned (column offsets and tuple widths are
// multiples of 4); an 8-byte key may straddle an 8-byte boundary.
__device__ __forceinline__ int64_t pg_load_key(const char* p, uint32_t bytes)
{
	if (bytes == 4) return (int64_t) *reinterpret_cast<const int32_t*>(p);
	if ((reinterpret_cast<uintptr_t>(p) & 7) == 0) return *reinterpret_cast<const int64_t*>(p);
	const uint32_t* q = reinterpret_cast<const uint32_t*>(p);
	return (int64_t) (((uint64_t) q[1] << 32) | q[0]);
}

// Bucket of one field value; mirrors the reference's arithmetic exactly,
// including its unsigned-int truncations.
__device__ __forceinline__ uint32_t pg_hash_field(const pg_hashfn& f, const char* p, uint32_t size)
{
	switch (f.fn) {
	case PG_FN_BYTES: {
		uint64_t h = 14695981039346656037ull;
		for (uint32_t i = 0; i < size; ++i) {
			h ^= (uint64_t) (int64_t) (signed char) p[i];
			h += (h << 1) + (h << 4) + (h << 5) + (h << 7) + (h << 8) + (h << 40);
		}
		return (uint32_t) (((h >> f.k) ^ h) & ((1ull << f.k) - 1));
	}
	case PG_FN_MIXRADIX:
		return (uint32_t) (pg_mix64((uint64_t) pg_load_key(p, size)) >> f.skipbits);
	case PG_FN_TPCHQ1MAGIC: {
		uint32_t v = *reinterpret_cast<const uint32_t*>(p);
		return (((v >> 4) | (v >> 16)) & 0x1u) | ((v >> 1) & 0x2u);
	}
	case PG_FN_ALWAYSZERO: return 0;
	default: break;
	}
	int64_t v = pg_load_key(p, size);
	switch (f.fn) {
	case PG_FN_MODULO: return (uint32_t) (v & f.k);
	case PG_FN_RANGE: {
		int64_t val = (int64_t) ((uint64_t) (v - f.min) << f.k);
		return (uint32_t) (val / (f.max - f.min + 1));
	}
	case PG_FN_EXACTRANGE: return (uint32_t) ((v - f.min) / f.bucketrange);
	case PG_FN_PARAMMODULO: return (uint32_t) (((v - f.min) & f.k) >> f.skipbits);
	case PG_FN_KNUTH:
		return (uint32_t) ((((uint64_t) v * 2654435761ull) & (uint64_t) f.k) >> f.skipbits);
	case PG_FN_TPCHORDERKEY: return (uint32_t) ((((v >> 2) & ~7LL) | (v & 7)) & f.k);
	case PG_FN_WILLIS: {
		uint64_t l = (uint64_t) v;
		l = ~l + (l << 21);
		l = (uint64_t) ((int64_t) l ^ ((int64_t) l >> 24));
		l = l + (l << 3) + (l << 8);
		l = (uint64_t) ((int64_t) l ^ ((int64_t) l >> 14));
		l = l + (l << 2) + (l << 4);
		l = (uint64_t) ((int64_t) l ^ ((int64_t) l >> 28));
		l = l + (l << 31);
		int64_t s = (int64_t) l;
		s = (s > 0) ? s : (int64_t) (0 - (uint64_t) s);
		return (uint32_t) (s & f.k);
	}
	default: return 0;
	}
}

// 64-bit finaliser of MurmurHash3 (Appleby): slot placement for the
// open-addressing tables. Bijective, so distinct keys never collide in full.
__device__ __forceinline__ uint64_t pg_mix64(uint64_t k)
{
	k ^= k >> 33; k *= 0xff51afd7ed558ccdull;
	k ^= k >> 33; k *= 0xc4ceb9fe1a85ec53ull;
	k ^= k >> 33;
	return k;
}

// Empty-slot marker of the open-addressing tables (all one bits, so a table
// clears with one memset). A real key equal to it takes a separate path.
#define PG_EMPTY_KEY ((long long) -1)

// Bounded spin budget for device-side waits (try_wait polls).
#define PG_SPIN_LIMIT (1u << 26)

__device__ __forceinline__ void pg_set_status(int* status, int code)
{
	atomicCAS(status, 0, code);
}

// ---------------------------------------------------------------------------
// PTX helpers: mbarrier + bulk (TMA) copies global -> shared
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t pg_smem_addr(const void* p)
{
	return (uint32_t) __cvta_generic_to_shared(p);
}

__device__ __forceinline__ void pg_mbar_init(uint64_t* bar, uint32_t count)
{
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(pg_smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void pg_fence_mbar_init()
{
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void pg_mbar_expect_tx(uint64_t* bar, uint32_t bytes)
{
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
			:: "r"(pg_smem_addr(bar)), "r"(bytes) : "memory");
}

// One-dimensional bulk copy (cp.async.bulk) of `bytes` (multiple of 16,
// both addresses 16-byte aligned) completing on `bar`.
__device__ __forceinline__ void pg_bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
			:: "r"(pg_smem_addr(dst)), "l"(src), "r"(bytes), "r"(pg_smem_addr(bar)) : "memory");
}

// Bulk copy global -> shared with an L2 eviction policy (streams: evict-first).
__device__ __forceinline__ void pg_bulk_g2s_hint(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
		uint64_t pol)
{
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
			" [%0], [%1], %2, [%3], %4;"
			:: "r"(pg_smem_addr(dst)), "l"(src), "r"(bytes), "r"(pg_smem_addr(bar)), "l"(pol) : "memory");
}

// Bounded wait for phase `parity` of `bar`. Returns false when it gave up.
__device__ __forceinline__ bool pg_mbar_wait(uint64_t* bar, uint32_t parity)
{
	uint32_t a = pg_smem_addr(bar);
	for (uint32_t it = 0; it < PG_SPIN_LIMIT; ++it) {
		uint32_t done;
		asm volatile("{\n\t.reg .pred p;\n\t"
				"mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
				"selp.u32 %0, 1, 0, p;\n\t}"
				: "=r"(done) : "r"(a), "r"(parity) : "memory");
		if (done) return true;
	}
	return false;
}

// Non-blocking test of phase `parity` of `bar`.
__device__ __forceinline__ bool pg_mbar_test(uint64_t* bar, uint32_t parity)
{
	uint32_t done;
	asm volatile("{\n\t.reg .pred p;\n\t"
			"mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
			"selp.u32 %0, 1, 0, p;\n\t}"
			: "=r"(done) : "r"(pg_smem_addr(bar)), "r"(parity) : "memory");
	return done != 0;
}

// The context's bounded-wait knob (PG_TUNE_SPIN_LIMIT), kept in word 1 of its
// device status block: 0 = the built-in limit. Kernels read it once.
__device__ __forceinline__ uint32_t pg_spin_knob(const int* status)
{
	return *reinterpret_cast<const volatile uint32_t*>(status + 1);
}

// Wait for a bulk copy's phase with the context's limit: `spin` = 0 polls with
// try_wait up to PG_SPIN_LIMIT times, else `spin` non-blocking tests. When the
// limit runs out the status word records PG_ERR_TIMEOUT and the wait goes on,
// bounded by PG_SPIN_LIMIT, until the copy has landed, so that no copy into
// shared memory outlives its wait (a buffer reused or a block exited with the
// copy in flight). False only when that drain also gave up.
__device__ __forceinline__ bool pg_mbar_wait_timed(uint64_t* bar, uint32_t parity, uint32_t spin, int* status)
{
	if (spin == 0) {
		if (pg_mbar_wait(bar, parity)) return true;
	} else {
		for (uint32_t i = 0; i < spin; ++i)
			if (pg_mbar_test(bar, parity)) return true;
	}
	pg_set_status(status, PG_ERR_TIMEOUT);
	return pg_mbar_wait(bar, parity);
}

// L2 cache policies (createpolicy): streams are evict-first so that the
// randomly accessed tables, loaded evict-last, stay resident in L2.
__device__ __forceinline__ uint64_t pg_policy_evict_first()
{
	uint64_t p;
	asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
	return p;
}

// Table-load policy: evict-last for `eighths`/8 of the accessed lines (the
// rest keep their priority), all lines when eighths is 0 or 8 or more.
__device__ __forceinline__ uint64_t pg_policy_keep(uint32_t eighths)
{
	uint64_t p;
	switch (eighths) {
	case 1: asm volatile("createpolicy.fractional.L2::evict_last.L2::evict_unchanged.b64 %0, 0.125;" : "=l"(p)); break;
	case 2: asm volatile("createpolicy.fractional.L2::evict_last.L2::evict_unchanged.b64 %0, 0.25;" : "=l"(p)); break;
	case 3: asm volatile("createpolicy.fractional.L2::evict_last.L2::evict_unchanged.b64 %0, 0.375;" : "=l"(p)); break;
	case 4: asm volatile("createpolicy.fractional.L2::evict_last.L2::evict_unchanged.b64 %0, 0.5;" : "=l"(p)); break;
	case 5: asm volatile("createpolicy.fractional.L2::evict_last.L2::evict_unchanged.b64 %0, 0.625;" : "=l"(p)); break;
	case 6: asm volatile("createpolicy.fractional.L2::evict_last.L2::evict_unchanged.b64 %0, 0.75;" : "=l"(p)); break;
	case 7: asm volatile("createpolicy.fractional.L2::evict_last.L2::evict_unchanged.b64 %0, 0.875;" : "=l"(p)); break;
	default: asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p)); break;
	}
	return p;
}

__device__ __forceinline__ uint64_t pg_policy_evict_normal()
{
	uint64_t p;
	asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
	return p;
}

__device__ __forceinline__ uint64_t pg_policy_evict_unchanged()
{
	uint64_t p;
	asm volatile("createpolicy.fractional.L2::evict_unchanged.b64 %0, 1.0;" : "=l"(p));
	return p;
}

__device__ __forceinline__ uint64_t pg_policy_evict_last()
{
	uint64_t p;
	asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
	return p;
}

__device__ __forceinline__ uint4 pg_ld_hint16(const void* p, uint64_t pol)
{
	uint4 v;
	asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
			: "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p), "l"(pol));
	return v;
}

__device__ __forceinline__ void pg_st_hint16(void* p, uint4 v, uint64_t pol)
{
	asm volatile("st.global.L1::no_allocate.L2::cache_hint.v4.u32 [%0], {%1,%2,%3,%4}, %5;"
			:: "l"(p), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "l"(pol) : "memory");
}

__device__ __forceinline__ uint4 pg_ld_stream16(const void* p) { return pg_ld_hint16(p, pg_policy_evict_first()); }
__device__ __forceinline__ uint4 pg_ld_table16(const void* p) { return pg_ld_hint16(p, pg_policy_evict_last()); }
__device__ __forceinline__ void pg_st_stream16(void* p, uint4 v) { pg_st_hint16(p, v, pg_policy_evict_first()); }

// 32-byte (256-bit) load of one table bucket, kept in L2 (evict-last).
struct pg_u64x4 { unsigned long long a, b, c, d; };
__device__ __forceinline__ pg_u64x4 pg_ld_bucket32(const void* p, uint64_t pol)
{
	pg_u64x4 v;
	asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u64 {%0,%1,%2,%3}, [%4], %5;"
			: "=l"(v.a), "=l"(v.b), "=l"(v.c), "=l"(v.d) : "l"(p), "l"(pol));
	return v;
}

// Bulk (TMA) store shared -> global; `bytes` a multiple of 16, both ends
// 16-byte aligned. Writers fence their shared stores to the async proxy first.
__device__ __forceinline__ void pg_fence_proxy_async_smem()
{
	asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void pg_bulk_s2g(void* dst, const void* src, uint32_t bytes)
{
	asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
			:: "l"(dst), "r"(pg_smem_addr(src)), "r"(bytes) : "memory");
	asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

__device__ __forceinline__ void pg_bulk_s2g_hint(void* dst, const void* src, uint32_t bytes, uint64_t pol)
{
	asm volatile("cp.async.bulk.global.shared::cta.bulk_group.L2::cache_hint [%0], [%1], %2, %3;"
			:: "l"(dst), "r"(pg_smem_addr(src)), "r"(bytes), "l"(pol) : "memory");
	asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}

// Waits until every committed bulk store has finished reading shared memory.
__device__ __forceinline__ void pg_bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// Waits until every committed bulk store has completed.
__device__ __forceinline__ void pg_bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

__host__ __device__ __forceinline__ uint64_t pg_div_up(uint64_t a, uint64_t b) { return (a + b - 1) / b; }
__host__ __device__ __forceinline__ uint64_t pg_min64(uint64_t a, uint64_t b) { return a < b ? a : b; }
__host__ __device__ __forceinline__ uint32_t pg_min32(uint32_t a, uint32_t b) { return a < b ? a : b; }

// Exclusive scan of n uint64 values in place on the device (multi-block).
int pg_scan_u64(pg_ctx* ctx, cudaStream_t s, uint64_t* data, uint64_t n, uint64_t* total_dev);

// Dec sums as exact fixed-point integers (pg_fixsum.h): order-independent,
// so a group's sum is the same on every run.
#include "pg_fixsum.h"

// The unit of one dec sum, in four device words made by pg_fx_prepare:
// p[0] the unit exponent s (a value is a count of units 2^s), p[1] the largest
// exponent field quantised, p[2] flags (PG_FX_RANGE: a value above that bound,
// the sum is redone with the exact bound; PG_FX_SPECIALS: infinities or NaNs,
// whose groups are patched afterwards), p[3] scratch. Kernels read s and the
// bound at their start, so no host round trip sits between the sampling pass
// and the aggregation.
struct PgFx {
	int* p;
};
#define PG_FX_RANGE 2u
#define PG_FX_SPECIALS 4u

// Quantises the dec value with bit pattern b for unit 2^s and bound `bound`.
// Values above the bound or not finite contribute 0 and set their flag in fl.
__device__ __forceinline__ pg_fx3 pg_fx_take(uint64_t b, int s, int bound, uint32_t& fl)
{
	const int e = pg_fx_field(b);
	if (e > bound) { fl |= e == PG_FX_EXP_SPECIAL ? PG_FX_SPECIALS : PG_FX_RANGE; return pg_fx3{0, 0, 0}; }
	return pg_fx_quant(b, s);
}

// The upper word of a value's count (sign extension) or of a sum's.
__device__ __forceinline__ uint64_t pg_fx_hi(const pg_fx3& a) { return (uint64_t) ((int64_t) a.w2 >> 63); }
__device__ __forceinline__ uint64_t pg_fx_hi(const pg_fx4& a) { return a.w3; }

// Adds count a into one group's table words (word k at t[k * stride]) with
// atomics (pg_fx_table_add). Returns whether the group's present marker is
// to be set (an add returned 0, or none was made).
__device__ __forceinline__ bool pg_fx_atomic_add(unsigned long long* t, uint64_t stride, const pg_fx4& a)
{
	return pg_fx_table_add(reinterpret_cast<uint64_t*>(t), stride, a, [](uint64_t* p, uint64_t v) {
		return (uint64_t) atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long) v);
	});
}

// Adds count a into a four-word chained table (pg_fx_chain_add) with atomics:
// for tables in shared memory.
__device__ __forceinline__ void pg_fx_atomic_chain_add(unsigned long long* t, uint64_t stride, const pg_fx4& a)
{
	pg_fx_chain_add(reinterpret_cast<uint64_t*>(t), stride, a, [](uint64_t* p, uint64_t v) {
		return (uint64_t) atomicAdd(reinterpret_cast<unsigned long long*>(p), (unsigned long long) v);
	});
}

// The same for ILP rows at once: word k of row j's group at base[slot[j] *
// sstride + k * wstride]. The low bits' chunks of the rows (values far below
// the column's largest) go to the lazy words first, with adds that return
// nothing; then the returning t2 adds of all rows are issued together, and
// each row reads its old t2 for the rare overflow into t3. So a row waits
// for one L2 round trip, with only its t2 part, old word and slot live across
// it. Rows with ok[j] false are skipped. With `present`, a row whose t2 add
// returned the initial 0 (or that made none) marks its slot present: a byte
// store per group rather than per row.
template <int ILP, class V>
__device__ __forceinline__ void pg_fx_atomic_add_rows(unsigned long long* base, uint64_t wstride,
		const uint64_t (&slot)[ILP], uint64_t sstride, const bool (&ok)[ILP], const V (&a)[ILP],
		unsigned char* present)
{
	#pragma unroll
	for (int j = 0; j < ILP; ++j) {
		if (!ok[j] || !(a[j].w0 | a[j].w1)) continue;
		#pragma unroll
		for (int k = 0; k < PG_FX_LAZY; ++k) {
			const uint64_t c = pg_fx_chunk(a[j].w0, a[j].w1, k);
			if (c) atomicAdd(&base[slot[j] * sstride + (PG_FX_L0 + k) * wstride], (unsigned long long) c);
		}
	}
	unsigned long long o[ILP];                              // old t2; 1 where no add was made
	#pragma unroll
	for (int j = 0; j < ILP; ++j)
		o[j] = ok[j] && a[j].w2 ? atomicAdd(&base[slot[j] * sstride + PG_FX_T2 * wstride], (unsigned long long) a[j].w2)
		                        : 1;
	#pragma unroll
	for (int j = 0; j < ILP; ++j) {
		if (!ok[j]) continue;
		int64_t r;
		uint64_t q;
		pg_fx_split_top(a[j].w2, pg_fx_hi(a[j]), r, q);
		if (r) q += pg_fx_overflow(o[j], r);
		if (q) atomicAdd(&base[slot[j] * sstride + PG_FX_T3 * wstride], (unsigned long long) q);
		if (present && (o[j] == 0 || !a[j].w2)) present[slot[j]] = 1;
	}
}

// Fills fx->p (16 bytes of device memory, allocated by the caller) for a dec
// sum over the 8-byte column at voff of n rows of width W: the largest finite
// exponent field over rows 0, step, 2 step, ..., widened by `margin` fields
// when sampled. Stream-ordered; no host round trip.
int pg_fx_prepare(pg_ctx* ctx, cudaStream_t s, const char* data, uint64_t n, uint32_t W, uint32_t voff,
		uint64_t step, int margin, PgFx fx);

// Patches the dec sums of groups that met infinities or NaNs: out holds
// ngroups rows (key of kbytes, 0 for no key, then the 8-byte sum) of the
// aggregation of `in` grouped on its key column.
int pg_fx_patch_specials(pg_ctx* ctx, cudaStream_t s, const pg_rel* in, uint32_t voff, char* out, uint64_t ngroups);

// Dense group table emission (pg_groupby.cu): acc holds a word per slot, or
// for a dec sum the PG_FX_WORDS table words of its count of units (fx), word
// k of slot i at acc[i + k * range].
int pg_dense_groups_emit(pg_ctx* ctx, cudaStream_t s, const unsigned long long* acc, PgFx fx,
		const unsigned char* present, uint64_t range, long long kmin, uint32_t kbytes, int val_type, int agg,
		void* out, uint64_t out_cap, unsigned long long* cursor);
