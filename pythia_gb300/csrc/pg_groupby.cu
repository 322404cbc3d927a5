// Group-by aggregation (aggregate_sum, aggregate_count) on sm_103a.
//
// Replaces GenericAggregate::remember + fold (operators/genericaggregate.cpp:
// 240-282; aggregatesum.cpp:53-107; aggregatecount.cpp:37-52) and the getNext
// emission of groups (genericaggregate.cpp:419-487). The reference keeps a
// chained table per thread (ThreadLocal) or one locked table (Global); a
// second aggregate over a merge combines thread partials.
//
// Here one open-addressing table per operator holds every group: the key word
// is claimed with atomicCAS, accumulators are updated with atomics. Integer
// sums and counts are exact (wrapping like the reference's CtInt/CtLong +=).
// Dec (double) sums are exact fixed-point integers (pg_fixsum.h): a value
// becomes a count of units 2^s, counts add into seven words per group with
// integer atomics (a value near the column's largest: one returning add, its
// old word giving the rare overflow into another word), and the sum is
// rounded to a double once at emission. Integer adds do not depend on the
// order in which threads arrive, so every run gives the same bits; when all
// values are within 2^135 of the largest, the result is the correctly rounded
// exact sum. The unit comes from the largest exponent of the column (sampled,
// with a margin, on large inputs; a value above the bound makes the operator
// redo the sum with the exact bound). Infinities and NaNs are summed on the
// side and patch their groups' results. Lanes of a warp that carry the same
// key are combined first (warp match), which cuts atomics on skewed keys;
// with few groups each CTA aggregates into a shared-memory table and merges
// once.
#include "pg_internal.cuh"
#include <algorithm>

#define GB_THREADS 256
#define GB_DEC (VT == PG_VAL_DEC && AGG == PG_AGG_SUM)     // inside templates on VT, AGG
#define GB_SMEM_SLOTS 4096

// An open-addressing group table. A group's aggregate is one word of acc (a
// count, a long sum, an int sum in its low 4 bytes) or, for a dec sum, the
// table words of its count of units (pg_fixsum.h) at acc[slot + k * (cap +
// 1)], k < PG_FX_WORDS.
struct GbTable {
	unsigned long long* keys;   // [cap + 1]; slot cap is the group whose key is the empty marker
	unsigned long long* acc;    // [PG_FX_WORDS (cap + 1)]
	int* sentinel_used;
	uint32_t log2cap;
	__device__ __forceinline__ uint64_t wstride() const { return (1ull << log2cap) + 1; }
};

// One row's (or a combined run's) value: an integer, or a dec sum's count.
struct GbVal {
	unsigned long long i;
	pg_fx4 f;
};

// Adds v into the aggregate of slot `slot` (a dec sum's word k at acc[slot +
// k * wstride]).
template <int VT, int AGG>
__device__ __forceinline__ void fold_slot(unsigned long long* acc, uint64_t wstride, uint64_t slot, const GbVal& v)
{
	if (AGG == PG_AGG_COUNT) atomicAdd(&acc[slot], v.i);
	else if (VT == PG_VAL_LONG) atomicAdd(&acc[slot], v.i);
	else if (VT == PG_VAL_INT) atomicAdd(reinterpret_cast<unsigned int*>(&acc[slot]), (unsigned int) v.i);
	else pg_fx_atomic_add(&acc[slot], wstride, v.f);
}

// A dec sum's count from table words acc[slot + k * wstride].
__device__ __forceinline__ pg_fx4 gb_table_count(const unsigned long long* acc, uint64_t wstride, uint64_t slot)
{
	return pg_fx_from_table(reinterpret_cast<const uint64_t*>(acc + slot), wstride);
}

// Loads one row's value (a dec value quantised for unit 2^fs, bound fb).
template <int VT, int AGG>
__device__ __forceinline__ GbVal gb_load_val(const char* r, uint32_t voff, int fs, int fb, uint32_t& fl)
{
	GbVal v = {0, {0, 0, 0, 0}};
	if (AGG == PG_AGG_COUNT) v.i = 1;
	else if (VT == PG_VAL_INT) v.i = (unsigned long long) (long long) *reinterpret_cast<const int32_t*>(r + voff);
	else if (VT == PG_VAL_LONG) v.i = (unsigned long long) pg_load_key(r + voff, 8);
	else v.f = pg_fx_widen(pg_fx_take((uint64_t) pg_load_key(r + voff, 8), fs, fb, fl));
	return v;
}

// Finds or claims the slot of key k. Returns cap (the side slot) for the
// empty-marker key, or UINT64_MAX when the table is full.
__device__ __forceinline__ uint64_t gb_slot(unsigned long long* keys, uint32_t log2cap, int64_t k,
		int* sentinel_used)
{
	const uint64_t cap = 1ull << log2cap, mask = cap - 1;
	if (k == PG_EMPTY_KEY) { if (!*sentinel_used) atomicExch(sentinel_used, 1); return cap; }
	uint64_t s = pg_mix64((uint64_t) k) >> (64 - log2cap);
	for (uint64_t probe = 0; probe < cap; ++probe) {
		unsigned long long cur = keys[s];
		if (cur == (unsigned long long) k) return s;
		if (cur == (unsigned long long) PG_EMPTY_KEY) {
			unsigned long long old = atomicCAS(&keys[s], (unsigned long long) PG_EMPTY_KEY, (unsigned long long) k);
			if (old == (unsigned long long) PG_EMPTY_KEY || old == (unsigned long long) k) return s;
		}
		s = (s + 1) & mask;
	}
	return UINT64_MAX;
}

// Combines the values of lanes in `peers` (same key) at the leader lane:
// integer adds (256-bit for dec sums' counts of units), exact in any order.
template <int VT, int AGG>
__device__ __forceinline__ void warp_combine(uint32_t peers, GbVal& v)
{
	GbVal t = {0, {0, 0, 0, 0}};
	uint32_t m = peers;
	while (m) {
		const int src = __ffs(m) - 1; m &= m - 1;
		if (GB_DEC) {
			const pg_fx4 x = {__shfl_sync(peers, v.f.w0, src), __shfl_sync(peers, v.f.w1, src),
			                  __shfl_sync(peers, v.f.w2, src), __shfl_sync(peers, v.f.w3, src)};
			pg_fx_add4(t.f, x);
		} else {
			t.i += __shfl_sync(peers, v.i, src);
		}
	}
	v = t;
}

template <int VT, int AGG, bool HASKEY, bool SMEM>
__global__ void __launch_bounds__(GB_THREADS)
k_gb_insert(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t koff, uint32_t kbytes,
		uint32_t voff, GbTable t, uint32_t smem_log2, PgFx fx, int* __restrict__ status)
{
	extern __shared__ __align__(16) unsigned char sm[];
	const uint32_t sc1 = SMEM ? (1u << smem_log2) + 1 : 0;
	unsigned long long* skeys = reinterpret_cast<unsigned long long*>(sm);
	unsigned long long* sacc = skeys + sc1;                 // [PG_FX_WORDS sc1]: a dec sum's words sc1 apart
	__shared__ int s_sentinel;
	if (SMEM) {
		for (uint32_t i = threadIdx.x; i < sc1; i += blockDim.x) skeys[i] = (unsigned long long) PG_EMPTY_KEY;
		for (uint32_t i = threadIdx.x; i < PG_FX_WORDS * sc1; i += blockDim.x) sacc[i] = 0;
		if (threadIdx.x == 0) s_sentinel = 0;
		__syncthreads();
	}
	bool full = false;
	uint32_t fl = 0;
	const int fs = GB_DEC ? fx.p[0] : 0, fb = GB_DEC ? fx.p[1] : 0;
	const int lane = threadIdx.x & 31;
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	const uint64_t n_round = pg_div_up(n, 32) * 32;
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n_round; i += stride) {
		bool valid = i < n;
		int64_t k = 0;
		GbVal v = {0, {0, 0, 0, 0}};
		if (valid) {
			const char* r = in + i * W;
			if (HASKEY) k = pg_load_key(r + koff, kbytes);
			v = gb_load_val<VT, AGG>(r, voff, fs, fb, fl);
		}
		// Lanes with the same key fold together first.
		uint32_t active = __ballot_sync(0xffffffffu, valid);
		if (!valid) continue;
		uint32_t peers = HASKEY ? __match_any_sync(active, (unsigned long long) k) : active;
		warp_combine<VT, AGG>(peers, v);
		if (lane != __ffs(peers) - 1) continue;
		if (SMEM) {
			uint64_t s = HASKEY ? gb_slot(skeys, smem_log2, k, &s_sentinel) : 0;
			if (s == UINT64_MAX) { full = true; continue; }
			fold_slot<VT, AGG>(sacc, sc1, s, v);
		} else {
			uint64_t s = HASKEY ? gb_slot(t.keys, t.log2cap, k, t.sentinel_used) : 0;
			if (s == UINT64_MAX) { full = true; continue; }
			fold_slot<VT, AGG>(t.acc, t.wstride(), s, v);
		}
	}
	if (full) pg_set_status(status, PG_ERR_TABLE_FULL);
	if (fl) atomicOr(reinterpret_cast<unsigned int*>(fx.p + 2), fl);
	if (SMEM) {
		// Merge this CTA's partial groups into the global table.
		__syncthreads();
		const uint32_t sc = 1u << smem_log2;
		for (uint32_t i = threadIdx.x; i <= sc; i += blockDim.x) {
			bool used = HASKEY ? ((i < sc) ? skeys[i] != (unsigned long long) PG_EMPTY_KEY : s_sentinel != 0)
			                   : i == 0;
			if (!used) continue;
			int64_t k = (i < sc) ? (int64_t) skeys[i] : PG_EMPTY_KEY;
			uint64_t s = HASKEY ? gb_slot(t.keys, t.log2cap, k, t.sentinel_used) : 0;
			if (s == UINT64_MAX) { pg_set_status(status, PG_ERR_TABLE_FULL); continue; }
			GbVal v = {sacc[i], {0, 0, 0, 0}};
			if (GB_DEC) v.f = gb_table_count(sacc, sc1, i);
			fold_slot<VT, AGG>(t.acc, t.wstride(), s, v);
		}
	}
}

// Global-table insert with four independent rows per thread per iteration:
// their key loads, slot reads and accumulator atomics are issued together, so
// the chains of dependent L2 round trips overlap instead of running one row
// at a time.
template <int VT, int AGG, bool MATCH, int GB_ILP>
__global__ void __launch_bounds__(GB_THREADS)
k_gb_insert_ilp(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t koff, uint32_t kbytes,
		uint32_t voff, GbTable t, PgFx fx, int* __restrict__ status)
{
	const uint64_t cap = 1ull << t.log2cap, mask = cap - 1;
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	const uint64_t step = stride * GB_ILP;
	bool full = false;
	uint32_t fl = 0;
	const int fs = GB_DEC ? fx.p[0] : 0, fb = GB_DEC ? fx.p[1] : 0;
	const int lane = threadIdx.x & 31;
	for (uint64_t base = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; base < pg_div_up(n, 32) * 32;
			base += step) {
		int64_t k[GB_ILP];
		GbVal v[GB_ILP];
		bool lead[GB_ILP];
		#pragma unroll
		for (int j = 0; j < GB_ILP; ++j) {
			const uint64_t i = base + j * stride;
			const bool valid = i < n;
			k[j] = 0; v[j] = GbVal{0, {0, 0, 0, 0}}; lead[j] = false;
			if (valid) {
				const char* r = in + i * W;
				k[j] = pg_load_key(r + koff, kbytes);
				v[j] = gb_load_val<VT, AGG>(r, voff, fs, fb, fl);
			}
			if (MATCH) {
				const uint32_t active = __ballot_sync(0xffffffffu, valid);
				if (valid) {
					const uint32_t peers = __match_any_sync(active, (unsigned long long) k[j]);
					warp_combine<VT, AGG>(peers, v[j]);
					lead[j] = lane == __ffs(peers) - 1;
				}
			} else {
				lead[j] = valid;
			}
		}
		uint64_t slot[GB_ILP];
		unsigned long long cur[GB_ILP];
		#pragma unroll
		for (int j = 0; j < GB_ILP; ++j) {
			if (!lead[j]) continue;
			if (k[j] == PG_EMPTY_KEY) { slot[j] = cap; cur[j] = 0; continue; }
			slot[j] = pg_mix64((uint64_t) k[j]) >> (64 - t.log2cap);
			cur[j] = t.keys[slot[j]];
		}
		#pragma unroll
		for (int j = 0; j < GB_ILP; ++j) {
			if (!lead[j]) continue;
			if (slot[j] == cap) { if (!*t.sentinel_used) atomicExch(t.sentinel_used, 1); continue; }
			uint64_t probe = 0;
			for (; probe < cap; ++probe) {
				if (cur[j] == (unsigned long long) k[j]) break;
				if (cur[j] == (unsigned long long) PG_EMPTY_KEY) {
					const unsigned long long old = atomicCAS(&t.keys[slot[j]], (unsigned long long) PG_EMPTY_KEY,
							(unsigned long long) k[j]);
					if (old == (unsigned long long) PG_EMPTY_KEY || old == (unsigned long long) k[j]) break;
					cur[j] = old;
					continue;
				}
				slot[j] = (slot[j] + 1) & mask;
				cur[j] = t.keys[slot[j]];
			}
			if (probe == cap) { full = true; lead[j] = false; }
		}
		if (GB_DEC) {
			pg_fx4 f[GB_ILP];
			#pragma unroll
			for (int j = 0; j < GB_ILP; ++j) f[j] = v[j].f;
			pg_fx_atomic_add_rows<GB_ILP>(t.acc, t.wstride(), slot, 1, lead, f, nullptr);
		} else {
			#pragma unroll
			for (int j = 0; j < GB_ILP; ++j)
				if (lead[j]) fold_slot<VT, AGG>(t.acc, 1, slot[j], v[j]);
		}
	}
	if (full) pg_set_status(status, PG_ERR_TABLE_FULL);
	if (fl) atomicOr(reinterpret_cast<unsigned int*>(fx.p + 2), fl);
}

// ---------------------------------------------------------------------------
// High-cardinality path: rows are first radix-partitioned on the top bits of
// the key mix (PG_FN_MIXRADIX) so that each partition holds about 1K groups;
// then one CTA per partition aggregates it in a shared-memory table with the
// same integer atomics, on shared instead of L2 atomics, and writes its
// groups out. A partition whose groups overflow the shared table sends the
// excess keys to the global table (emitted afterwards).
// ---------------------------------------------------------------------------
#define GBP_THREADS 512
// Slots of a partition's shared-memory table: 4096 (64 KB, three CTAs per
// SM), or 2048 for dec sums (key and the four words of the chained form,
// pg_fx_chain_add: 80 KB, two CTAs per SM); a partition holds about 1K groups
// either way.
#define GBP_SLOTS (GB_DEC ? 2048u : 4096u)
#define GBP_GROUPS 1024u

// Slot of key k in a per-partition table: low bits of the mix (the top bits
// are the partition number).
template <uint32_t SLOTS>
__device__ __forceinline__ uint32_t gbp_slot(unsigned long long* keys, int64_t k, int* sentinel)
{
	if (k == PG_EMPTY_KEY) { if (!*sentinel) atomicExch(sentinel, 1); return SLOTS; }
	uint32_t s = (uint32_t) (pg_mix64((uint64_t) k) & (SLOTS - 1));
	for (uint32_t probe = 0; probe < SLOTS; ++probe) {
		const unsigned long long cur = keys[s];
		if (cur == (unsigned long long) k) return s;
		if (cur == (unsigned long long) PG_EMPTY_KEY) {
			const unsigned long long old = atomicCAS(&keys[s], (unsigned long long) PG_EMPTY_KEY, (unsigned long long) k);
			if (old == (unsigned long long) PG_EMPTY_KEY || old == (unsigned long long) k) return s;
		}
		s = (s + 1) & (SLOTS - 1);
	}
	return UINT32_MAX;
}

// Writes one group's row: kbytes of key (none for 0), then its aggregate:
// word a, or for a dec sum the count c of units 2^fx_s rounded to a double.
template <int VT, int AGG>
__device__ __forceinline__ void gb_write_agg(char* o, uint32_t kbytes, int64_t k, unsigned long long a,
		const pg_fx4& c, int fx_s)
{
	if (kbytes == 4) *reinterpret_cast<int32_t*>(o) = (int32_t) k;
	else if (kbytes == 8) {
		reinterpret_cast<uint32_t*>(o)[0] = (uint32_t) k;
		reinterpret_cast<uint32_t*>(o)[1] = (uint32_t) ((uint64_t) k >> 32);
	}
	o += kbytes;
	if (AGG == PG_AGG_SUM && VT == PG_VAL_INT) { *reinterpret_cast<uint32_t*>(o) = (uint32_t) a; return; }
	if (GB_DEC) a = (unsigned long long) __double_as_longlong(pg_fx_double4(c, fx_s));
	reinterpret_cast<uint32_t*>(o)[0] = (uint32_t) a;
	reinterpret_cast<uint32_t*>(o)[1] = (uint32_t) (a >> 32);
}

template <int VT, int AGG, bool MATCH>
__global__ void __launch_bounds__(GBP_THREADS)
k_gb_part_agg(const char* __restrict__ rows, const uint64_t* __restrict__ offs, uint32_t P, uint32_t W,
		uint32_t koff, uint32_t kbytes, uint32_t voff, GbTable t, PgFx fx, char* __restrict__ out, uint64_t out_cap,
		unsigned long long* __restrict__ cursor, int* __restrict__ overflow, int* __restrict__ status)
{
	extern __shared__ __align__(16) unsigned char sm[];
	constexpr uint32_t SW = GBP_SLOTS + 1;                                         // a dec sum's word stride
	unsigned long long* skeys = reinterpret_cast<unsigned long long*>(sm);        // [SLOTS + 1]
	unsigned long long* sacc = skeys + SW;                                         // [SLOTS + 1], 4 [SLOTS + 1] for dec
	__shared__ int s_sent;
	__shared__ uint32_t wtot[GBP_THREADS / 32];
	__shared__ unsigned long long s_base;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const uint32_t ow = kbytes + ((AGG == PG_AGG_SUM && VT == PG_VAL_INT) ? 4 : 8);
	uint32_t fl = 0;
	const int fs = GB_DEC ? fx.p[0] : 0, fb = GB_DEC ? fx.p[1] : 0;
	for (uint32_t part = blockIdx.x; part < P; part += gridDim.x) {
		for (uint32_t i = tid; i <= GBP_SLOTS; i += blockDim.x) {
			skeys[i] = (unsigned long long) PG_EMPTY_KEY; sacc[i] = 0;
			if (GB_DEC) { sacc[i + SW] = 0; sacc[i + 2 * SW] = 0; sacc[i + 3 * SW] = 0; }
		}
		if (tid == 0) s_sent = 0;
		__syncthreads();
		const uint64_t lo = offs[part], hi = offs[part + 1];
		bool spilled = false;
		for (uint64_t i = lo + tid; i < lo + pg_div_up(hi - lo, 32) * 32; i += blockDim.x) {
			const bool valid = i < hi;
			int64_t k = 0;
			GbVal v = {0, {0, 0, 0, 0}};
			if (valid) {
				const char* r = rows + i * W;
				k = pg_load_key(r + koff, kbytes);
				v = gb_load_val<VT, AGG>(r, voff, fs, fb, fl);
			}
			if (MATCH) {
				const uint32_t active = __ballot_sync(0xffffffffu, valid);
				if (!valid) continue;
				const uint32_t peers = __match_any_sync(active, (unsigned long long) k);
				warp_combine<VT, AGG>(peers, v);
				if (lane != __ffs(peers) - 1) continue;
			} else if (!valid) {
				continue;
			}
			const uint32_t s = gbp_slot<GBP_SLOTS>(skeys, k, &s_sent);
			if (s != UINT32_MAX) {
				if (GB_DEC) pg_fx_atomic_chain_add(&sacc[s], SW, v.f);
				else fold_slot<VT, AGG>(sacc, SW, s, v);
				continue;
			}
			// Shared table full: this key lives in the global table.
			const uint64_t g = gb_slot(t.keys, t.log2cap, k, t.sentinel_used);
			if (g == UINT64_MAX) { pg_set_status(status, PG_ERR_TABLE_FULL); continue; }
			fold_slot<VT, AGG>(t.acc, t.wstride(), g, v);
			spilled = true;
		}
		if (spilled) atomicExch(overflow, 1);
		__syncthreads();
		// Emit: count used slots per thread, scan, reserve, write.
		uint32_t mine = 0;
		for (uint32_t i = tid; i <= GBP_SLOTS; i += blockDim.x)
			mine += (i < GBP_SLOTS) ? (skeys[i] != (unsigned long long) PG_EMPTY_KEY) : (s_sent != 0);
		uint32_t x = mine;
		#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
			if (lane >= o) x += y;
		}
		if (lane == 31) wtot[warp] = x;
		__syncthreads();
		uint32_t before = 0, total = 0;
		for (int w = 0; w < GBP_THREADS / 32; ++w) { const uint32_t c = wtot[w]; before += w < warp ? c : 0; total += c; }
		if (tid == 0) s_base = total ? atomicAdd(cursor, (unsigned long long) total) : 0;
		__syncthreads();
		uint64_t pos = s_base + before + x - mine;
		for (uint32_t i = tid; i <= GBP_SLOTS; i += blockDim.x) {
			const bool used = (i < GBP_SLOTS) ? (skeys[i] != (unsigned long long) PG_EMPTY_KEY) : (s_sent != 0);
			if (!used) continue;
			if (pos < out_cap)
				gb_write_agg<VT, AGG>(out + pos * ow, kbytes, i < GBP_SLOTS ? (int64_t) skeys[i] : PG_EMPTY_KEY,
						sacc[i], GB_DEC ? pg_fx_from_chain(reinterpret_cast<const uint64_t*>(sacc + i), SW)
						                : pg_fx4{0, 0, 0, 0}, fs);
			++pos;
		}
		__syncthreads();
	}
	if (fl) atomicOr(reinterpret_cast<unsigned int*>(fx.p + 2), fl);
}

template <int VT, int AGG, bool HASKEY>
__global__ void k_gb_emit(GbTable t, uint32_t kbytes, char* __restrict__ out, uint64_t cap_rows,
		unsigned long long* __restrict__ cursor, uint64_t nonkey_rows, PgFx fx)
{
	const int fx_s = GB_DEC ? fx.p[0] : 0;
	const uint64_t cap = 1ull << t.log2cap;
	const uint32_t aw = (AGG == PG_AGG_SUM && VT == PG_VAL_INT) ? 4 : 8;
	const uint32_t ow = (HASKEY ? kbytes : 0) + aw;
	const uint64_t limit = HASKEY ? cap + 1 : 1;
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < pg_div_up(limit, 32) * 32;
			i += (uint64_t) gridDim.x * blockDim.x) {
		bool used = false;
		if (i < limit) {
			if (!HASKEY) used = nonkey_rows > 0;
			else if (i < cap) used = t.keys[i] != (unsigned long long) PG_EMPTY_KEY;
			else used = *t.sentinel_used != 0;
		}
		uint32_t ball = __ballot_sync(0xffffffffu, used);
		if (!ball) continue;
		int lane = threadIdx.x & 31;
		unsigned long long base = 0;
		if (lane == __ffs(ball) - 1) base = atomicAdd(cursor, (unsigned long long) __popc(ball));
		base = __shfl_sync(0xffffffffu, base, __ffs(ball) - 1);
		if (!used) continue;
		uint64_t pos = base + __popc(ball & ((1u << lane) - 1));
		if (pos >= cap_rows) continue;
		const int64_t k = HASKEY ? (i < cap ? (int64_t) t.keys[i] : PG_EMPTY_KEY) : 0;
		gb_write_agg<VT, AGG>(out + pos * ow, HASKEY ? kbytes : 0, k, t.acc[i],
				GB_DEC ? gb_table_count(t.acc, t.wstride(), i) : pg_fx4{0, 0, 0, 0}, fx_s);
	}
}

// ---------------------------------------------------------------------------
// Dense key domain (keys span at most a few times the group count, e.g.
// group numbers 0..G-1 or surrogate keys): a min/max pass, then the slot of a
// row is key - kmin. No probing and no key words: a row costs its atomics
// (one for a typical dec value, as for the integer aggregates) and, for
// sums, a byte store marking the group present. A dec sum's table keeps
// each of its PG_FX_WORDS words in an array of its own (word k of slot i at
// acc[i + k * range]), so the word every row adds into takes 8 bytes a group
// of L2.
// ---------------------------------------------------------------------------
// Min and max key over rows 0, step, 2 step, ... (step 1: every row).
template <bool VEC16>
__global__ void k_gb_key_minmax(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t koff,
		uint32_t kbytes, unsigned long long* __restrict__ mm, uint64_t step)
{
	unsigned long long lo = ~0ull, hi = 0;
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	const uint64_t ns = pg_div_up(n, step);
	for (uint64_t j = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; j < ns; j += stride) {
		const uint64_t i = j * step;
		int64_t k;
		if (VEC16) {
			const uint4 t = __ldg(reinterpret_cast<const uint4*>(in) + i);
			k = koff == 0 ? (int64_t) (((uint64_t) t.y << 32) | t.x) : (int64_t) (((uint64_t) t.w << 32) | t.z);
		} else {
			k = pg_load_key(in + i * W + koff, kbytes);
		}
		const unsigned long long u = (unsigned long long) k ^ (1ull << 63);
		lo = u < lo ? u : lo;
		hi = u > hi ? u : hi;
	}
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		const unsigned long long a = __shfl_down_sync(0xffffffffu, lo, o), b = __shfl_down_sync(0xffffffffu, hi, o);
		lo = a < lo ? a : lo;
		hi = b > hi ? b : hi;
	}
	if ((threadIdx.x & 31) == 0) { atomicMin(&mm[0], lo); atomicMax(&mm[1], hi); }
}

// Key and value words of row i: the 8-byte key at koff and the value at voff
// (an int sign-extended), from one 16-byte load when VEC16.
template <int VT, bool VEC16>
__device__ __forceinline__ void gb_row_kv(const char* __restrict__ in, uint64_t i, uint32_t W, uint32_t koff,
		uint32_t kbytes, uint32_t voff, int64_t& k, uint64_t& vbits)
{
	if (VEC16) {
		const uint4 t = __ldg(reinterpret_cast<const uint4*>(in) + i);
		k = koff == 0 ? (int64_t) (((uint64_t) t.y << 32) | t.x) : (int64_t) (((uint64_t) t.w << 32) | t.z);
		vbits = voff == 0 ? (((uint64_t) t.y << 32) | t.x) : voff == 8 ? (((uint64_t) t.w << 32) | t.z)
			: voff == 4 ? t.y : t.w;
		if (VT == PG_VAL_INT) vbits = (uint64_t) (int64_t) (int32_t) (voff == 0 ? t.x : voff == 4 ? t.y : voff == 8 ? t.z : t.w);
	} else {
		const char* r = in + i * W;
		k = pg_load_key(r + koff, kbytes);
		vbits = VT == PG_VAL_INT ? (uint64_t) (int64_t) *reinterpret_cast<const int32_t*>(r + voff)
			: (uint64_t) pg_load_key(r + voff, 8);
	}
}

#define GBD_ILP 4
// ILP rows per thread in flight (their loads and atomics issued together).
template <int VT, int AGG, bool VEC16, int ILP>
__global__ void __launch_bounds__(GB_THREADS)
k_gb_dense(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t koff, uint32_t kbytes, uint32_t voff,
		long long kmin, uint64_t range, unsigned long long* __restrict__ acc, PgFx fx,
		unsigned char* __restrict__ present, unsigned int* __restrict__ overflow)
{
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	bool outside = false;
	uint32_t fl = 0;
	const int fs = GB_DEC ? fx.p[0] : 0, fb = GB_DEC ? fx.p[1] : 0;
	for (uint64_t base = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; base < n; base += stride * ILP) {
		uint64_t d[ILP];
		unsigned long long iv[ILP];
		pg_fx3 f[ILP];
		bool ok[ILP];
		#pragma unroll
		for (int j = 0; j < ILP; ++j) {
			const uint64_t i = base + j * stride;
			ok[j] = i < n;
			d[j] = 0; iv[j] = 0; f[j] = pg_fx3{0, 0, 0};
			if (!ok[j]) continue;
			int64_t k;
			uint64_t vbits;
			gb_row_kv<VT, VEC16>(in, i, W, koff, kbytes, voff, k, vbits);
			d[j] = (uint64_t) k - (uint64_t) kmin;
			if (d[j] >= range) { ok[j] = false; outside = true; d[j] = 0; continue; }   // key outside the table
			if (AGG == PG_AGG_COUNT) iv[j] = 1;
			else if (GB_DEC) f[j] = pg_fx_take(vbits, fs, fb, fl);
			else iv[j] = vbits;
		}
		if (GB_DEC) {
			pg_fx_atomic_add_rows<ILP>(acc, range, d, 1, ok, f, present);
		} else {
			#pragma unroll
			for (int j = 0; j < ILP; ++j) {
				if (!ok[j]) continue;
				if (VT == PG_VAL_INT && AGG == PG_AGG_SUM)
					atomicAdd(reinterpret_cast<unsigned int*>(&acc[d[j]]), (unsigned int) iv[j]);
				else atomicAdd(&acc[d[j]], iv[j]);
				if (AGG == PG_AGG_SUM) present[d[j]] = 1;
			}
		}
	}
	if (outside) *overflow = 1;
	if (fl) atomicOr(reinterpret_cast<unsigned int*>(fx.p + 2), fl);
}

// Dense group-by over a window of at most GBS_MAX_SLOTS keys: each CTA sums
// its rows into a copy of the table in shared memory (dec sums' seven table
// words, int sums in the low 4 bytes, counts and long sums in 8), then adds
// each slot it saw into the global table once. Few groups otherwise put every
// row's atomic on a handful of L2 lines.
#define GBS_MAX_SLOTS 4096
#define GBS_MAX_SLOTS_DEC 1536                     // 57 bytes a slot: two CTAs per SM
template <int VT, int AGG, bool VEC16>
__global__ void __launch_bounds__(GB_THREADS)
k_gb_dense_smem(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t koff, uint32_t kbytes, uint32_t voff,
		long long kmin, uint32_t range, unsigned long long* __restrict__ acc, PgFx fx,
		unsigned char* __restrict__ present, unsigned int* __restrict__ overflow)
{
	constexpr uint32_t SW = GB_DEC ? PG_FX_WORDS : 1;                                 // shared words per slot
	extern __shared__ __align__(16) unsigned char gsm[];
	unsigned long long* const sacc = reinterpret_cast<unsigned long long*>(gsm);
	unsigned char* const spres = gsm + (size_t) range * SW * 8;
	for (uint32_t i = threadIdx.x; i < range * SW; i += blockDim.x) sacc[i] = 0;
	for (uint32_t i = threadIdx.x; i < range; i += blockDim.x) spres[i] = 0;
	__syncthreads();
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	bool outside = false;
	uint32_t fl = 0;
	const int fs = GB_DEC ? fx.p[0] : 0, fb = GB_DEC ? fx.p[1] : 0;
	for (uint64_t base = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; base < n; base += stride * GBD_ILP) {
		uint32_t d[GBD_ILP];
		unsigned long long iv[GBD_ILP];
		pg_fx3 f[GBD_ILP];
		bool ok[GBD_ILP];
		#pragma unroll
		for (int j = 0; j < GBD_ILP; ++j) {
			const uint64_t i = base + j * stride;
			ok[j] = i < n;
			d[j] = 0; iv[j] = 0; f[j] = pg_fx3{0, 0, 0};
			if (!ok[j]) continue;
			int64_t k;
			uint64_t vbits;
			gb_row_kv<VT, VEC16>(in, i, W, koff, kbytes, voff, k, vbits);
			const uint64_t dd = (uint64_t) k - (uint64_t) kmin;
			if (dd >= range) { ok[j] = false; outside = true; continue; }   // key outside the table
			d[j] = (uint32_t) dd;
			if (AGG == PG_AGG_COUNT) iv[j] = 1;
			else if (GB_DEC) f[j] = pg_fx_take(vbits, fs, fb, fl);
			else iv[j] = vbits;
		}
		#pragma unroll
		for (int j = 0; j < GBD_ILP; ++j) {
			if (!ok[j]) continue;
			if (GB_DEC) pg_fx_atomic_add(&sacc[d[j]], range, pg_fx_widen(f[j]));
			else if (VT == PG_VAL_INT && AGG == PG_AGG_SUM)
				atomicAdd(reinterpret_cast<unsigned int*>(&sacc[d[j]]), (unsigned int) iv[j]);
			else atomicAdd(&sacc[d[j]], iv[j]);
			if (AGG == PG_AGG_SUM) spres[d[j]] = 1;
		}
	}
	if (outside) *overflow = 1;
	if (fl) atomicOr(reinterpret_cast<unsigned int*>(fx.p + 2), fl);
	__syncthreads();
	for (uint32_t i = threadIdx.x; i < range; i += blockDim.x) {
		if (AGG == PG_AGG_COUNT) {
			if (sacc[i]) atomicAdd(&acc[i], sacc[i]);
			continue;
		}
		if (!spres[i]) continue;
		if (GB_DEC) pg_fx_atomic_add(&acc[i], range, gb_table_count(sacc, range, i));
		else if (VT == PG_VAL_INT) atomicAdd(reinterpret_cast<unsigned int*>(&acc[i]), (unsigned int) sacc[i]);
		else atomicAdd(&acc[i], sacc[i]);
		present[i] = 1;
	}
}

template <int VT, int AGG>
__global__ void k_gb_dense_emit(const unsigned long long* __restrict__ acc, PgFx fx,
		const unsigned char* __restrict__ present, uint64_t range, long long kmin, uint32_t kbytes,
		char* __restrict__ out, uint64_t cap_rows, unsigned long long* __restrict__ cursor)
{
	const int fx_s = GB_DEC ? fx.p[0] : 0;
	const uint32_t aw = (AGG == PG_AGG_SUM && VT == PG_VAL_INT) ? 4 : 8;
	const uint32_t ow = kbytes + aw;
	const int lane = threadIdx.x & 31;
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < pg_div_up(range, 32) * 32;
			i += (uint64_t) gridDim.x * blockDim.x) {
		const bool used = i < range && (AGG == PG_AGG_COUNT ? acc[i] != 0 : present[i] != 0);
		const uint32_t ball = __ballot_sync(0xffffffffu, used);
		if (!ball) continue;
		unsigned long long base = 0;
		if (lane == 0) base = atomicAdd(cursor, (unsigned long long) __popc(ball));
		base = __shfl_sync(0xffffffffu, base, 0);
		if (!used) continue;
		const uint64_t pos = base + __popc(ball & ((1u << lane) - 1));
		if (pos >= cap_rows) continue;
		const int64_t k = (int64_t) ((uint64_t) kmin + i);
		if (GB_DEC)
			gb_write_agg<VT, AGG>(out + pos * ow, kbytes, k, 0, gb_table_count(acc, range, i), fx_s);
		else gb_write_agg<VT, AGG>(out + pos * ow, kbytes, k, acc[i], pg_fx4{0, 0, 0, 0}, 0);
	}
}

// ---------------------------------------------------------------------------
// Dec sums: the unit, and the groups that met infinities or NaNs
// ---------------------------------------------------------------------------
// Largest finite exponent field of the 8-byte column at voff over rows 0,
// step, 2 step, ... into p[3].
__global__ void k_fx_max_field(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t voff, uint64_t step,
		int* __restrict__ p)
{
	int m = 0;
	const uint64_t ns = pg_div_up(n, step);
	for (uint64_t j = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; j < ns; j += (uint64_t) gridDim.x * blockDim.x) {
		const int e = pg_fx_field((uint64_t) pg_load_key(in + j * step * W + voff, 8));
		if (e != PG_FX_EXP_SPECIAL && e > m) m = e;
	}
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
	if ((threadIdx.x & 31) == 0 && m) atomicMax(&p[3], m);
}

// p[0] unit exponent, p[1] bound, p[2] flags cleared, from the field in p[3].
__global__ void k_fx_finish(int* __restrict__ p, int margin)
{
	const int bound = min(p[3] + margin, PG_FX_EXP_SPECIAL - 1);
	p[0] = pg_fx_unit(bound);
	p[1] = bound;
	p[2] = 0;
}

int pg_fx_prepare(pg_ctx* ctx, cudaStream_t s, const char* data, uint64_t n, uint32_t W, uint32_t voff,
		uint64_t step, int margin, PgFx fx)
{
	PG_CUDA(ctx, cudaMemsetAsync(fx.p, 0, 16, s));
	if (n) {
		const int blocks = (int) std::max<uint64_t>(1, std::min<uint64_t>(pg_div_up(pg_div_up(n, step), 256),
				(uint64_t) ctx->sm_count * 8));
		k_fx_max_field<<<blocks, 256, 0, s>>>(data, n, W, voff, step, fx.p);
		PG_LAUNCHED(ctx);
	}
	k_fx_finish<<<1, 1, 0, s>>>(fx.p, step > 1 ? margin : 0);
	PG_LAUNCHED(ctx);
	return PG_OK;
}

// Rows whose dec value is an infinity or NaN, counted.
__global__ void k_fx_special_count(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t voff,
		unsigned long long* __restrict__ cnt)
{
	unsigned long long c = 0;
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x)
		c += pg_fx_field((uint64_t) pg_load_key(in + i * W + voff, 8)) == PG_FX_EXP_SPECIAL;
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
	if ((threadIdx.x & 31) == 0 && c) atomicAdd(cnt, c);
}

// The special values of each group that has any, OR-ed into fl[slot] of a
// small table of their keys (all rows key 0 when kbytes is 0).
__global__ void k_fx_special_collect(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t koff,
		uint32_t kbytes, uint32_t voff, unsigned long long* __restrict__ keys, unsigned int* __restrict__ fl,
		uint32_t log2cap, int* __restrict__ sentinel)
{
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x) {
		const uint64_t b = (uint64_t) pg_load_key(in + i * W + voff, 8);
		if (pg_fx_field(b) != PG_FX_EXP_SPECIAL) continue;
		const int64_t k = kbytes ? pg_load_key(in + i * W + koff, kbytes) : 0;
		const uint64_t slot = gb_slot(keys, log2cap, k, sentinel);
		if (slot != UINT64_MAX) atomicOr(&fl[slot], pg_fx_special(b));
	}
}

// Output rows (key of kbytes, then the 8-byte sum) of groups in the table get
// the IEEE result of their special values.
__global__ void k_fx_special_patch(char* __restrict__ out, uint64_t rows, uint32_t kbytes,
		const unsigned long long* __restrict__ keys, const unsigned int* __restrict__ fl, uint32_t log2cap,
		const int* __restrict__ sentinel)
{
	const uint64_t cap = 1ull << log2cap;
	for (uint64_t r = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; r < rows; r += (uint64_t) gridDim.x * blockDim.x) {
		char* o = out + r * (kbytes + 8);
		int64_t k = 0;
		if (kbytes == 4) k = *reinterpret_cast<const int32_t*>(o);
		else if (kbytes == 8)
			k = (int64_t) (((uint64_t) reinterpret_cast<const uint32_t*>(o)[1] << 32) | reinterpret_cast<const uint32_t*>(o)[0]);
		uint64_t slot = UINT64_MAX;
		if (k == PG_EMPTY_KEY) { if (*sentinel) slot = cap; }
		else {
			uint64_t h = pg_mix64((uint64_t) k) >> (64 - log2cap);
			for (uint64_t probe = 0; probe < cap; ++probe, h = (h + 1) & (cap - 1)) {
				if (keys[h] == (unsigned long long) k) { slot = h; break; }
				if (keys[h] == (unsigned long long) PG_EMPTY_KEY) break;
			}
		}
		if (slot == UINT64_MAX || !fl[slot]) continue;
		const uint64_t v = pg_fx_special_bits(fl[slot]);
		reinterpret_cast<uint32_t*>(o + kbytes)[0] = (uint32_t) v;
		reinterpret_cast<uint32_t*>(o + kbytes)[1] = (uint32_t) (v >> 32);
	}
}

int pg_fx_patch_specials(pg_ctx* ctx, cudaStream_t s, const pg_rel* in, uint32_t voff, char* out, uint64_t ngroups)
{
	int rc;
	unsigned long long* cnt = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &cnt, 16))) return rc;
	PG_CUDA(ctx, cudaMemsetAsync(cnt, 0, 16, s));
	const int blocks = (int) std::max<uint64_t>(1, std::min<uint64_t>(pg_div_up(in->n, 256), (uint64_t) ctx->sm_count * 8));
	k_fx_special_count<<<blocks, 256, 0, s>>>((const char*) in->data, in->n, in->width, voff, cnt);
	PG_LAUNCHED(ctx);
	unsigned long long h = 0;
	PG_CUDA(ctx, cudaMemcpyAsync(&h, cnt, 8, cudaMemcpyDeviceToHost, s));
	PG_CUDA(ctx, cudaStreamSynchronize(s));
	pg_free_async(ctx, s, cnt);
	if (!h || !ngroups) return PG_OK;
	uint32_t lg = 6;
	while ((1ull << lg) < 2 * h) ++lg;
	const uint64_t cap = 1ull << lg;
	char* mem = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &mem, (cap + 1) * 12 + 16))) return rc;
	unsigned long long* keys = reinterpret_cast<unsigned long long*>(mem);
	unsigned int* fl = reinterpret_cast<unsigned int*>(keys + cap + 1);
	int* sentinel = reinterpret_cast<int*>(fl + cap + 1);
	PG_CUDA(ctx, cudaMemsetAsync(keys, 0xFF, (cap + 1) * 8, s));
	PG_CUDA(ctx, cudaMemsetAsync(fl, 0, (cap + 1) * 4 + 8, s));
	k_fx_special_collect<<<blocks, 256, 0, s>>>((const char*) in->data, in->n, in->width, in->key_off, in->key_bytes,
			voff, keys, fl, lg, sentinel);
	PG_LAUNCHED(ctx);
	const int pblocks = (int) std::max<uint64_t>(1, std::min<uint64_t>(pg_div_up(ngroups, 256), (uint64_t) ctx->sm_count * 8));
	k_fx_special_patch<<<pblocks, 256, 0, s>>>(out, ngroups, in->key_bytes, keys, fl, lg, sentinel);
	PG_LAUNCHED(ctx);
	pg_free_async(ctx, s, mem);
	return PG_OK;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
// One dense aggregation over the key window [kmin, kmin + range): table, fill,
// aggregation, emission. *overflow: some key lay outside the window (nothing
// of this run is usable then); *fxfl: the dec sum's flags (fx).
template <int VT, int AGG>
static int gb_dense_window(pg_ctx* ctx, cudaStream_t s, const pg_rel* in, uint32_t voff, bool vec16, long long kmin,
		uint64_t range, void* out, uint64_t out_cap, uint64_t* ngroups, bool* overflow, PgFx fx, uint32_t* fxfl)
{
	int rc;
	char* mem = nullptr;
	const uint64_t words = range * (GB_DEC ? PG_FX_WORDS : 1);
	const size_t bytes = words * 8 + range + 128;
	if ((rc = pg_alloc_async(ctx, s, (void**) &mem, bytes))) return rc;
	unsigned long long* acc = reinterpret_cast<unsigned long long*>(mem);      // a dec sum: word k of slot i at acc[i + k range]
	unsigned long long* cursor = acc + words;
	unsigned char* present = reinterpret_cast<unsigned char*>(cursor + 1);
	unsigned int* oflag = reinterpret_cast<unsigned int*>((reinterpret_cast<uintptr_t>(present + range) + 15) & ~uintptr_t(15));
	PG_CUDA(ctx, cudaMemsetAsync(mem, 0, bytes, s));
	if (range <= (GB_DEC ? GBS_MAX_SLOTS_DEC : GBS_MAX_SLOTS) && ctx->tune[PG_TUNE_GROUPBY_PATH] != 7) {
		// Few groups: per-CTA tables in shared memory, one flush each.
		const int sbytes = (int) (range * (GB_DEC ? 8 * PG_FX_WORDS + 1 : 9));
		int per_sm = 0;
		if (vec16) {
			PG_CUDA(ctx, cudaFuncSetAttribute(k_gb_dense_smem<VT, AGG, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sbytes));
			PG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gb_dense_smem<VT, AGG, true>, GB_THREADS, sbytes));
		} else {
			PG_CUDA(ctx, cudaFuncSetAttribute(k_gb_dense_smem<VT, AGG, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sbytes));
			PG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gb_dense_smem<VT, AGG, false>, GB_THREADS, sbytes));
		}
		const int sblocks = (int) std::min<uint64_t>(pg_div_up(in->n, (uint64_t) GB_THREADS * GBD_ILP),
				(uint64_t) ctx->sm_count * std::max(per_sm, 1));
		if (vec16) k_gb_dense_smem<VT, AGG, true><<<sblocks, GB_THREADS, sbytes, s>>>((const char*) in->data, in->n,
				in->width, in->key_off, in->key_bytes, voff, kmin, (uint32_t) range, acc, fx, present, oflag);
		else k_gb_dense_smem<VT, AGG, false><<<sblocks, GB_THREADS, sbytes, s>>>((const char*) in->data, in->n,
				in->width, in->key_off, in->key_bytes, voff, kmin, (uint32_t) range, acc, fx, present, oflag);
		PG_LAUNCHED(ctx);
	} else {
		// Rows in flight per thread: eight for counts and integer sums, four for
		// dec sums, whose kernel holds more registers a row (85 at eight rows:
		// 3.60 against 2.74 ms at four for 256M rows in 1M groups).
		const int64_t knob = ctx->tune[PG_TUNE_GROUPBY_ILP];
		const int ilp = knob == 4 ? GBD_ILP : knob == 8 ? 8 : GB_DEC ? GBD_ILP : 8;
		const int gblocks = (int) std::min<uint64_t>(pg_div_up(in->n, (uint64_t) GB_THREADS * ilp),
				(uint64_t) ctx->sm_count * 8);
#define GBD_LAUNCH(V, I) k_gb_dense<VT, AGG, V, I><<<gblocks, GB_THREADS, 0, s>>>((const char*) in->data, in->n, \
				in->width, in->key_off, in->key_bytes, voff, kmin, range, acc, fx, present, oflag)
		if (vec16 && ilp == 8) GBD_LAUNCH(true, 8);
		else if (vec16) GBD_LAUNCH(true, GBD_ILP);
		else if (ilp == 8) GBD_LAUNCH(false, 8);
		else GBD_LAUNCH(false, GBD_ILP);
#undef GBD_LAUNCH
		PG_LAUNCHED(ctx);
	}
	const int eblocks = (int) std::min<uint64_t>(pg_div_up(range, 256), (uint64_t) ctx->sm_count * 8);
	k_gb_dense_emit<VT, AGG><<<eblocks, 256, 0, s>>>(acc, fx, present, range, kmin, in->key_bytes, (char*) out,
			out_cap, cursor);
	PG_LAUNCHED(ctx);
	unsigned long long h[2] = {0, 0};
	unsigned int f = 0;
	PG_CUDA(ctx, cudaMemcpyAsync(&h[0], cursor, 8, cudaMemcpyDeviceToHost, s));
	PG_CUDA(ctx, cudaMemcpyAsync(&h[1], oflag, 4, cudaMemcpyDeviceToHost, s));
	if (GB_DEC) PG_CUDA(ctx, cudaMemcpyAsync(&f, fx.p + 2, 4, cudaMemcpyDeviceToHost, s));
	PG_CUDA(ctx, cudaStreamSynchronize(s));
	pg_free_async(ctx, s, mem);
	*ngroups = h[0];
	*overflow = (h[1] & 0xFFFFFFFFull) != 0;
	*fxfl |= f;
	return PG_OK;
}

// Key range of rows 0, step, 2 step, ...: h[0], h[1] = min and max with the
// sign bit flipped (unsigned order = signed order).
static int gb_key_range(pg_ctx* ctx, cudaStream_t s, const pg_rel* in, bool vec16, uint64_t step, unsigned long long* h)
{
	int rc;
	unsigned long long* mm = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &mm, 32))) return rc;
	const unsigned long long init[2] = {~0ull, 0ull};
	PG_CUDA(ctx, cudaMemcpyAsync(mm, init, 16, cudaMemcpyHostToDevice, s));
	const uint64_t ns = pg_div_up(in->n, step);
	const int blocks = (int) std::max<uint64_t>(1, std::min<uint64_t>(pg_div_up(ns, 256), (uint64_t) ctx->sm_count * 8));
	if (vec16) k_gb_key_minmax<true><<<blocks, 256, 0, s>>>((const char*) in->data, in->n, in->width, in->key_off,
			in->key_bytes, mm, step);
	else k_gb_key_minmax<false><<<blocks, 256, 0, s>>>((const char*) in->data, in->n, in->width, in->key_off,
			in->key_bytes, mm, step);
	PG_LAUNCHED(ctx);
	PG_CUDA(ctx, cudaMemcpyAsync(h, mm, 16, cudaMemcpyDeviceToHost, s));
	PG_CUDA(ctx, cudaStreamSynchronize(s));
	pg_free_async(ctx, s, mm);
	return PG_OK;
}

// Dense keys: slot = key - kmin. Large inputs first try a key window from a
// sample of every 1024th row widened by an eighth on each side (no full
// min/max pass); a key outside it sends the operator to the exact window.
template <int VT, int AGG>
static int gb_dense(pg_ctx* ctx, cudaStream_t s, const pg_rel* in, uint32_t voff, uint64_t hint,
		void* out, uint64_t out_cap, uint64_t* ngroups, bool* done, PgFx fx, uint32_t* fxfl)
{
	*done = false;
	int rc;
	const bool vec16 = in->width == 16 && (in->key_off == 0 || in->key_off == 8) && in->key_bytes == 8 &&
		(reinterpret_cast<uintptr_t>(in->data) & 15) == 0 &&
		(AGG == PG_AGG_COUNT || (VT == PG_VAL_INT ? (voff & 3) == 0 : (voff == 0 || voff == 8)));
	const uint64_t limit = std::max<uint64_t>(4 * std::max<uint64_t>(hint, 1), std::min<uint64_t>(2 * in->n, 1ull << 22));
	unsigned long long h[2];
	if (in->n >= (1ull << 22)) {
		if ((rc = gb_key_range(ctx, s, in, vec16, 1024, h))) return rc;
		const unsigned long long span = h[1] - h[0];
		const unsigned long long slack = span / 8 + 64;
		const unsigned long long lo_u = h[0] > slack ? h[0] - slack : 0;
		const unsigned long long hi_u = ~0ull - h[1] > slack ? h[1] + slack : ~0ull;
		const uint64_t range = hi_u - lo_u + 1;
		if (range != 0 && range <= limit && range <= (1ull << 28)) {
			bool overflow = false;
			if ((rc = gb_dense_window<VT, AGG>(ctx, s, in, voff, vec16, (long long) (lo_u ^ (1ull << 63)), range,
					out, out_cap, ngroups, &overflow, fx, fxfl))) return rc;
			if (!overflow) {
				*done = true;
				if (*ngroups > out_cap) return pg_fail(ctx, PG_ERR_OUTPUT_FULL, "pg_groupby: output capacity too small");
				return pg_check_status(ctx, s, "pg_groupby");
			}
		}
	}
	if ((rc = gb_key_range(ctx, s, in, vec16, 1, h))) return rc;
	const long long kmin = (long long) (h[0] ^ (1ull << 63)), kmax = (long long) (h[1] ^ (1ull << 63));
	const uint64_t range = (uint64_t) kmax - (uint64_t) kmin + 1;
	if (range == 0 || range > limit || range > (1ull << 28)) return PG_OK;
	bool overflow = false;
	if ((rc = gb_dense_window<VT, AGG>(ctx, s, in, voff, vec16, kmin, range, out, out_cap, ngroups, &overflow,
			fx, fxfl))) return rc;
	*done = true;
	if (*ngroups > out_cap) return pg_fail(ctx, PG_ERR_OUTPUT_FULL, "pg_groupby: output capacity too small");
	return pg_check_status(ctx, s, "pg_groupby");
}

template <int VT, int AGG>
static int gb_run(pg_ctx* ctx, cudaStream_t s, const pg_rel* in, uint32_t voff, uint64_t hint,
		void* out, uint64_t out_cap, uint64_t* ngroups, PgFx fx, uint32_t* fxfl)
{
	const bool haskey = in->key_bytes != 0;
	const int64_t gpath = ctx->tune[PG_TUNE_GROUPBY_PATH];
	if (haskey && in->n && (gpath == 0 || gpath == 6 || gpath == 7)) {
		bool done = false;
		int rc = gb_dense<VT, AGG>(ctx, s, in, voff, hint, out, out_cap, ngroups, &done, fx, fxfl);
		if (rc || done) return rc;
	}
	uint64_t groups = haskey ? std::max<uint64_t>(1, std::min<uint64_t>(hint ? hint : in->n, in->n ? in->n : 1)) : 1;
	for (int attempt = 0; attempt < 6; ++attempt) {
		uint32_t lg = 10;
		while ((1ull << lg) < 2 * groups) ++lg;
		const uint64_t cap = 1ull << lg;
		GbTable t;
		t.log2cap = lg;
		char* mem = nullptr;
		int rc;
		size_t bytes = (cap + 1) * 8 * (1 + PG_FX_WORDS) + 64;
		if ((rc = pg_alloc_async(ctx, s, (void**) &mem, bytes))) return rc;
		t.keys = reinterpret_cast<unsigned long long*>(mem);
		t.acc = t.keys + cap + 1;
		t.sentinel_used = reinterpret_cast<int*>(t.acc + PG_FX_WORDS * (cap + 1));
		unsigned long long* cursor = reinterpret_cast<unsigned long long*>(t.sentinel_used + 2);
		PG_CUDA(ctx, cudaMemsetAsync(t.keys, 0xFF, (cap + 1) * 8, s));
		PG_CUDA(ctx, cudaMemsetAsync(t.acc, 0, (cap + 1) * 8 * PG_FX_WORDS + 64, s));
		const bool smem = groups <= GB_SMEM_SLOTS / (GB_DEC ? 8 : 2);       // tables up to 66 KB
		// Path knob: 0 by size, 1 global table (warp-combined), 2 partitioned,
		// 3 global table without the warp combine.
		const int64_t path = ctx->tune[PG_TUNE_GROUPBY_PATH];
		const bool part_ok = haskey && !smem && in->n < (1ull << 32) && in->width <= 1024;
		unsigned int f = 0;
		if (part_ok && (path == 2 || path == 4 || (path == 0 && in->n >= 4 * groups))) {
			// High cardinality: partition by key hash, aggregate per partition.
			uint32_t lp = 1;
			while ((1ull << lp) < groups / GBP_GROUPS && lp < 12) ++lp;
			const uint32_t P = 1u << lp;
			char* prow = nullptr;
			uint64_t* poffs = nullptr;
			int* oflag = reinterpret_cast<int*>(cursor + 1);
			if ((rc = pg_alloc_async(ctx, s, (void**) &prow, in->n * in->width))) return rc;
			if ((rc = pg_alloc_async(ctx, s, (void**) &poffs, (P + 1) * 8))) return rc;
			pg_hashfn fn;
			fn.fn = PG_FN_MIXRADIX; fn.k = 0; fn.min = 0; fn.max = 0; fn.bucketrange = 0;
			fn.skipbits = 64 - lp; fn.nbuckets = P;
			if ((rc = pg_partition_fn(ctx, s, in, fn, prow, poffs))) return rc;
			const size_t psm = (size_t) (GBP_SLOTS + 1) * (GB_DEC ? 40 : 16);
			const int pblocks = (int) std::min<uint64_t>(P, (uint64_t) ctx->sm_count * (GB_DEC ? 2 : 3));   // CTAs per SM
			if (path == 4) {
				PG_CUDA(ctx, cudaFuncSetAttribute(k_gb_part_agg<VT, AGG, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) psm));
				k_gb_part_agg<VT, AGG, false><<<pblocks, GBP_THREADS, psm, s>>>(prow, poffs, P, in->width, in->key_off,
						in->key_bytes, voff, t, fx, (char*) out, out_cap, cursor, oflag, ctx->d_status);
			} else {
				PG_CUDA(ctx, cudaFuncSetAttribute(k_gb_part_agg<VT, AGG, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) psm));
				k_gb_part_agg<VT, AGG, true><<<pblocks, GBP_THREADS, psm, s>>>(prow, poffs, P, in->width, in->key_off,
						in->key_bytes, voff, t, fx, (char*) out, out_cap, cursor, oflag, ctx->d_status);
			}
			PG_LAUNCHED(ctx);
			int hflag = 0;
			PG_CUDA(ctx, cudaMemcpyAsync(&hflag, oflag, 4, cudaMemcpyDeviceToHost, s));
			rc = pg_check_status(ctx, s, "pg_groupby");
			pg_free_async(ctx, s, prow);
			pg_free_async(ctx, s, poffs);
			if (rc == PG_ERR_TABLE_FULL) { pg_free_async(ctx, s, mem); groups *= 4; continue; }
			if (rc) { pg_free_async(ctx, s, mem); return rc; }
			if (hflag) {   // groups that overflowed a partition's table
				int eblocks = (int) std::min<uint64_t>(pg_div_up(cap + 1, 256), (uint64_t) ctx->sm_count * 8);
				k_gb_emit<VT, AGG, true><<<eblocks, 256, 0, s>>>(t, in->key_bytes, (char*) out, out_cap, cursor, 0, fx);
				PG_LAUNCHED(ctx);
			}
			unsigned long long ng = 0;
			PG_CUDA(ctx, cudaMemcpyAsync(&ng, cursor, 8, cudaMemcpyDeviceToHost, s));
			if (GB_DEC) PG_CUDA(ctx, cudaMemcpyAsync(&f, fx.p + 2, 4, cudaMemcpyDeviceToHost, s));
			PG_CUDA(ctx, cudaStreamSynchronize(s));
			pg_free_async(ctx, s, mem);
			*ngroups = ng;
			*fxfl |= f;
			if (ng > out_cap) return pg_fail(ctx, PG_ERR_OUTPUT_FULL, "pg_groupby: output capacity too small");
			return PG_OK;
		}
		uint32_t slg = 1;
		while ((1u << slg) < 2 * groups) ++slg;
		if (!haskey) slg = 0;
		const size_t smem_bytes = smem ? ((size_t) (1u << slg) + 1) * 8 * (1 + PG_FX_WORDS) : 0;
		int blocks = (int) std::min<uint64_t>(pg_div_up(std::max<uint64_t>(in->n, 1), GB_THREADS),
				(uint64_t) ctx->sm_count * (smem ? 4 : 8));
		if (in->n) {
			#define GB_LAUNCH(HK, SM) cudaFuncSetAttribute(k_gb_insert<VT, AGG, HK, SM>, \
					cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem_bytes); \
					k_gb_insert<VT, AGG, HK, SM><<<blocks, GB_THREADS, smem_bytes, s>>>( \
					(const char*) in->data, in->n, in->width, in->key_off, in->key_bytes, voff, t, slg, fx, ctx->d_status)
			if (haskey && smem) { GB_LAUNCH(true, true); }
			else if (haskey && (path == 3 || path == 5)) {
				if (path == 5)
					k_gb_insert_ilp<VT, AGG, false, 8><<<blocks, GB_THREADS, 0, s>>>((const char*) in->data, in->n,
							in->width, in->key_off, in->key_bytes, voff, t, fx, ctx->d_status);
				else
					k_gb_insert_ilp<VT, AGG, false, 4><<<blocks, GB_THREADS, 0, s>>>((const char*) in->data, in->n,
							in->width, in->key_off, in->key_bytes, voff, t, fx, ctx->d_status);
			}
			else if (haskey) {
				k_gb_insert_ilp<VT, AGG, true, 4><<<blocks, GB_THREADS, 0, s>>>((const char*) in->data, in->n,
						in->width, in->key_off, in->key_bytes, voff, t, fx, ctx->d_status);
			}
			else { GB_LAUNCH(false, true); }
			#undef GB_LAUNCH
			PG_LAUNCHED(ctx);
		}
		rc = pg_check_status(ctx, s, "pg_groupby");
		if (rc == PG_ERR_TABLE_FULL) { pg_free_async(ctx, s, mem); groups *= 4; continue; }
		if (rc) { pg_free_async(ctx, s, mem); return rc; }
		int eblocks = (int) std::min<uint64_t>(pg_div_up(cap + 1, 256), (uint64_t) ctx->sm_count * 8);
		if (haskey) k_gb_emit<VT, AGG, true><<<eblocks, 256, 0, s>>>(t, in->key_bytes, (char*) out, out_cap, cursor, 0, fx);
		else k_gb_emit<VT, AGG, false><<<1, 32, 0, s>>>(t, 0, (char*) out, out_cap, cursor, in->n, fx);
		PG_LAUNCHED(ctx);
		unsigned long long ng = 0;
		PG_CUDA(ctx, cudaMemcpyAsync(&ng, cursor, 8, cudaMemcpyDeviceToHost, s));
		if (GB_DEC) PG_CUDA(ctx, cudaMemcpyAsync(&f, fx.p + 2, 4, cudaMemcpyDeviceToHost, s));
		PG_CUDA(ctx, cudaStreamSynchronize(s));
		pg_free_async(ctx, s, mem);
		*ngroups = ng;
		*fxfl |= f;
		if (ng > out_cap) return pg_fail(ctx, PG_ERR_OUTPUT_FULL, "pg_groupby: output capacity too small");
		return PG_OK;
	}
	return pg_fail(ctx, PG_ERR_TABLE_FULL, "pg_groupby: group table kept overflowing");
}

// A dec sum: the unit from the column's largest exponent (every 1024th row
// with a margin of 4x on large inputs), the aggregation, a rerun on the exact
// unit if a value lay above the sampled bound, then the groups that met
// infinities or NaNs patched.
static int gb_dec_sum(pg_ctx* ctx, cudaStream_t s, const pg_rel* in, uint32_t voff, uint64_t hint,
		void* out, uint64_t out_cap, uint64_t* ngroups)
{
	int rc;
	PgFx fx;
	if ((rc = pg_alloc_async(ctx, s, (void**) &fx.p, 16))) return rc;
	const bool sampled = in->n >= (1ull << 22);
	uint32_t fl = 0;
	rc = pg_fx_prepare(ctx, s, (const char*) in->data, in->n, in->width, voff, sampled ? 1024 : 1, 2, fx);
	if (!rc) rc = gb_run<PG_VAL_DEC, PG_AGG_SUM>(ctx, s, in, voff, hint, out, out_cap, ngroups, fx, &fl);
	if (!rc && (fl & PG_FX_RANGE)) {
		fl = 0;
		rc = pg_fx_prepare(ctx, s, (const char*) in->data, in->n, in->width, voff, 1, 0, fx);
		if (!rc) rc = gb_run<PG_VAL_DEC, PG_AGG_SUM>(ctx, s, in, voff, hint, out, out_cap, ngroups, fx, &fl);
	}
	if (!rc && (fl & PG_FX_SPECIALS)) rc = pg_fx_patch_specials(ctx, s, in, voff, (char*) out, *ngroups);
	pg_free_async(ctx, s, fx.p);
	return rc;
}

extern "C" int pg_groupby(pg_ctx* ctx, pg_stream stream, const pg_rel* in,
		uint32_t val_off, int val_type, int agg, uint64_t groups_hint,
		void* out, uint64_t out_capacity, uint64_t* ngroups)
{
	if (!ctx || !in || !ngroups) return pg_fail(ctx, PG_ERR_ARG, "pg_groupby: null argument");
	if (in->n && !in->data) return pg_fail(ctx, PG_ERR_ARG, "pg_groupby: null data");
	if (in->width == 0 || (in->width & 3)) return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_groupby: tuple width must be a multiple of 4");
	if (in->key_bytes != 0 && ((in->key_bytes != 4 && in->key_bytes != 8) || (in->key_off & 3) ||
			in->key_off + in->key_bytes > in->width))
		return pg_fail(ctx, PG_ERR_ARG, "pg_groupby: key must be a 4-byte-aligned int or long column, or absent");
	if (agg != PG_AGG_SUM && agg != PG_AGG_COUNT) return pg_fail(ctx, PG_ERR_ARG, "pg_groupby: bad aggregate");
	if (agg == PG_AGG_SUM) {
		uint32_t vb = val_type == PG_VAL_INT ? 4 : 8;
		if (val_type < 0 || val_type > 2 || (val_off & 3) || val_off + vb > in->width)
			return pg_fail(ctx, PG_ERR_ARG, "pg_groupby: bad sum column");
	}
	cudaStream_t s = (cudaStream_t) stream;
	const PgFx none = {nullptr};
	uint32_t fl = 0;
	if (agg == PG_AGG_COUNT)
		return gb_run<PG_VAL_LONG, PG_AGG_COUNT>(ctx, s, in, val_off, groups_hint, out, out_capacity, ngroups, none, &fl);
	if (val_type == PG_VAL_INT)
		return gb_run<PG_VAL_INT, PG_AGG_SUM>(ctx, s, in, val_off, groups_hint, out, out_capacity, ngroups, none, &fl);
	if (val_type == PG_VAL_LONG)
		return gb_run<PG_VAL_LONG, PG_AGG_SUM>(ctx, s, in, val_off, groups_hint, out, out_capacity, ngroups, none, &fl);
	return gb_dec_sum(ctx, s, in, val_off, groups_hint, out, out_capacity, ngroups);
}

// Emits the present groups of a dense group table (acc/present over `range`
// slots, group key = kmin + slot) as (key, agg) rows of kbytes + agg bytes,
// appending at *cursor. Used by pg_hashjoin_groupby.
int pg_dense_groups_emit(pg_ctx* ctx, cudaStream_t s, const unsigned long long* acc, PgFx fx,
		const unsigned char* present, uint64_t range, long long kmin, uint32_t kbytes, int val_type, int agg,
		void* out, uint64_t out_cap, unsigned long long* cursor)
{
	const int eblocks = (int) std::min<uint64_t>(pg_div_up(range, 256), (uint64_t) ctx->sm_count * 8);
	if (agg == PG_AGG_COUNT)
		k_gb_dense_emit<PG_VAL_LONG, PG_AGG_COUNT><<<eblocks, 256, 0, s>>>(acc, fx, present, range, kmin, kbytes, (char*) out, out_cap, cursor);
	else if (val_type == PG_VAL_INT)
		k_gb_dense_emit<PG_VAL_INT, PG_AGG_SUM><<<eblocks, 256, 0, s>>>(acc, fx, present, range, kmin, kbytes, (char*) out, out_cap, cursor);
	else if (val_type == PG_VAL_LONG)
		k_gb_dense_emit<PG_VAL_LONG, PG_AGG_SUM><<<eblocks, 256, 0, s>>>(acc, fx, present, range, kmin, kbytes, (char*) out, out_cap, cursor);
	else
		k_gb_dense_emit<PG_VAL_DEC, PG_AGG_SUM><<<eblocks, 256, 0, s>>>(acc, fx, present, range, kmin, kbytes, (char*) out, out_cap, cursor);
	PG_LAUNCHED(ctx);
	return PG_OK;
}
