// Hash join build and probe on sm_103a.
//
// Replaces HashJoinOp (operators/join.cpp:273-675) and its chained-bucket
// HashTable (util/hashtable.{h,cpp}). The reference hashes the build key into
// a bucket, takes the bucket's spinlock, appends the sbuild tuple (key +
// build-projected columns, join.cpp:641-667), and later walks the chain per
// probe tuple (join.cpp:503-562), emitting constructOutputTuple
// (join.cpp:475-501) for every key match.
//
// Here the table is open addressing with linear probing over 16-byte slots
// {int64 key, uint64 value}: inserts claim a slot with one 64-bit atomicCAS on
// the key word; the value is the build-projected columns packed into 8 bytes
// when they fit, else the build row index (the output then gathers from R).
// Keys equal to the empty marker live in a small side list. Duplicate build
// keys are legal (each occupies its own slot); the build records whether any
// occurred, and the probe takes a single-pass path when keys are unique
// (PK-FK joins) and a count-then-write path otherwise.
//
// Probe (unique keys): each CTA takes tiles of 2048 probe tuples, loads them
// with streaming (evict-first) 16-byte loads, probes the table with
// evict-last loads so the table stays in L2, ranks matches with warp ballots
// in tile order, reserves one output range per tile with a single atomicAdd,
// and writes coalesced rows. With PG_JOIN_COUNT/SUM the matches are folded
// into a count and a wrapping int64 sum instead (aggregate_count /
// aggregate_sum over the join, aggregatecount.cpp:37-52,
// aggregatesum.cpp:81-107).
#include "pg_internal.cuh"
#include "pg_hashtable.cuh"
#include "pg_pred.cuh"
#include <algorithm>
#include <vector>

#define HJ_THREADS 256
#define HJ_ITEMS 8
#define HJ_TILE (HJ_THREADS * HJ_ITEMS)
#define HJ_SIDE_CAP0 1024

struct HjCols {                 // projected columns, in projection order
	int n;
	int ow_words;               // output width in 4-byte words
	uint8_t side[HJ_MAX_COLS];  // 0 build, 1 probe
	uint16_t src[HJ_MAX_COLS];  // word offset: probe tuple, packed build value, or build tuple
	uint8_t words[HJ_MAX_COLS];
};

struct HjProbeTable {
	const unsigned long long* slots;   // hashed: 2 words per slot
	uint32_t log2cap;
	const unsigned long long* side;    // values of build keys equal to the empty marker
	uint32_t nside;
	const unsigned long long* dense_val;   // dense: value per key - dmin
	const uint32_t* dense_bits;            // dense: presence bit per key - dmin
	const uint32_t* dense32;               // narrow dense: value - vmin, or all ones
	unsigned long long vmin;
	long long dmin;
	unsigned long long drange;
	uint32_t cache;                        // L2 policy knob: bits 0-1 table loads (0 evict-last,
	                                       // 1 normal, 2 unchanged, 3 first); bit 2 probe reads,
	                                       // bit 3 output stores normal instead of evict-first;
	                                       // bits 4-6 evict-last for that many eighths of the
	                                       // table's lines (0: all); bit 7 table loads kept in L1
	const HjDenseHdr* hdr;                 // speculative narrow dense table: window and checks, else null
};


// First slot of key k's probe sequence: always even, so the sequence starts
// at a 32-byte bucket of two slots that one 256-bit load fetches.
__device__ __forceinline__ uint64_t hj_slot0(int64_t k, uint32_t log2cap)
{
	return (pg_mix64((uint64_t) k) >> (65 - log2cap)) << 1;
}

__device__ __forceinline__ uint32_t hj_word(const char* tuple, uint32_t w)
{
	return reinterpret_cast<const uint32_t*>(tuple)[w];
}

// The packed value's word positions in a build tuple of any width as one
// word: bits 0-1 the word count (0..2), bits 2-9 and 10-17 the two word
// indices. Read in the kernel without an indexed local array.
static uint32_t hj_pack_code(const HjBuildCols& bc)
{
	uint32_t code = 0, o = 0;
	for (int c = 0; c < bc.n; ++c)
		for (int j = 0; j < bc.words[c] && o < 2; ++j, ++o) code |= (uint32_t) ((bc.roff[c] + j) & 255) << (2 + 8 * o);
	return code | o;
}

__device__ __forceinline__ uint64_t hj_pack(const char* t, uint32_t code)
{
	const uint32_t nw = code & 3;
	uint64_t v = 0;
	if (nw > 0) v = hj_word(t, (code >> 2) & 255);
	if (nw > 1) v |= (uint64_t) hj_word(t, (code >> 10) & 255) << 32;
	return v;
}

// Open-addressing build: each thread inserts HT_ILP tuples at once. Their
// key loads and their atomicCAS on the slots' key words are issued together,
// and each tuple then walks on to the next slot only when its slot was taken,
// so the L2 round trips of several inserts overlap instead of running one
// tuple at a time. A key already present is inserted again (duplicates are
// kept) and flags the table as not unique.
#define HT_ILP 4
__global__ void __launch_bounds__(256)
k_ht_build(const char* __restrict__ R, uint64_t n, uint32_t W, uint32_t koff,
		uint32_t kbytes, uint32_t pcode, bool inline_val, unsigned long long* __restrict__ slots,
		uint32_t log2cap, unsigned long long* __restrict__ side, uint32_t side_cap,
		unsigned int* __restrict__ side_count, int* __restrict__ flags, int* __restrict__ status)
{
	const uint64_t mask = (1ull << log2cap) - 1;
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	bool dup = false, full = false;
	for (uint64_t base = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; base < n; base += stride * HT_ILP) {
		int64_t k[HT_ILP];
		uint64_t v[HT_ILP], s[HT_ILP], tries[HT_ILP];
		bool act[HT_ILP];
		#pragma unroll
		for (int j = 0; j < HT_ILP; ++j) {
			const uint64_t i = base + j * stride;
			act[j] = i < n;
			k[j] = 0; v[j] = 0; s[j] = 0; tries[j] = 0;
			if (!act[j]) continue;
			const char* t = R + i * W;
			k[j] = pg_load_key(t + koff, kbytes);
			v[j] = inline_val ? hj_pack(t, pcode) : i;
			if (k[j] == PG_EMPTY_KEY) {
				const unsigned int idx = atomicAdd(side_count, 1u);
				if (idx < side_cap) side[idx] = v[j]; else atomicOr(flags, 2);
				act[j] = false;
				continue;
			}
			s[j] = hj_slot0(k[j], log2cap);
		}
		for (;;) {
			bool any = false;
			unsigned long long old[HT_ILP];
			#pragma unroll
			for (int j = 0; j < HT_ILP; ++j)
				if (act[j]) old[j] = atomicCAS(&slots[2 * s[j]], (unsigned long long) PG_EMPTY_KEY, (unsigned long long) k[j]);
			#pragma unroll
			for (int j = 0; j < HT_ILP; ++j) {
				if (!act[j]) continue;
				if (old[j] == (unsigned long long) PG_EMPTY_KEY) { slots[2 * s[j] + 1] = v[j]; act[j] = false; continue; }
				if ((long long) old[j] == k[j]) dup = true;
				s[j] = (s[j] + 1) & mask;
				if (++tries[j] > mask) { full = true; act[j] = false; continue; }
				any = true;
			}
			if (!any) break;
		}
	}
	if (full) pg_set_status(status, PG_ERR_TABLE_FULL);
	if (__any_sync(__activemask(), dup) && dup) atomicOr(flags, 1);
}

// Key range of the build side (signed keys mapped to ordered unsigned words)
// and the range of the packed build values (unsigned): mm = {kmin, kmax, vmin, vmax}.
__device__ __forceinline__ uint64_t hj_pack_value(const char* t, const HjBuildCols& bc)
{
	uint32_t w[2] = {0, 0};
	int o = 0;
	for (int c = 0; c < bc.n; ++c)
		for (int j = 0; j < bc.words[c]; ++j) w[o++] = reinterpret_cast<const uint32_t*>(t)[bc.roff[c] + j];
	return ((uint64_t) w[1] << 32) | w[0];
}

__global__ void k_key_minmax(const char* __restrict__ R, uint64_t n, uint32_t W, uint32_t koff,
		uint32_t kbytes, HjBuildCols bc, unsigned long long* __restrict__ mm)
{
	unsigned long long lo = ~0ull, hi = 0, vlo = ~0ull, vhi = 0;
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
			i += (uint64_t) gridDim.x * blockDim.x) {
		const char* t = R + i * W;
		const unsigned long long u = (unsigned long long) pg_load_key(t + koff, kbytes) ^ (1ull << 63);
		const unsigned long long v = hj_pack_value(t, bc);
		lo = u < lo ? u : lo;
		hi = u > hi ? u : hi;
		vlo = v < vlo ? v : vlo;
		vhi = v > vhi ? v : vhi;
	}
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		unsigned long long a = __shfl_down_sync(0xffffffffu, lo, o), b = __shfl_down_sync(0xffffffffu, hi, o);
		unsigned long long c = __shfl_down_sync(0xffffffffu, vlo, o), d = __shfl_down_sync(0xffffffffu, vhi, o);
		lo = a < lo ? a : lo;
		hi = b > hi ? b : hi;
		vlo = c < vlo ? c : vlo;
		vhi = d > vhi ? d : vhi;
	}
	if ((threadIdx.x & 31) == 0) {
		atomicMin(&mm[0], lo); atomicMax(&mm[1], hi);
		atomicMin(&mm[2], vlo); atomicMax(&mm[3], vhi);
	}
}

// Narrow dense table: entry key - dmin holds value - vmin; an entry that was
// not all ones before the exchange means a duplicate key.
__global__ void k_dense32_build(const char* __restrict__ R, uint64_t n, uint32_t W, uint32_t koff,
		uint32_t kbytes, HjBuildCols bc, long long dmin, unsigned long long vmin,
		uint32_t* __restrict__ table, int* __restrict__ flags)
{
	bool dup = false;
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
			i += (uint64_t) gridDim.x * blockDim.x) {
		const char* t = R + i * W;
		const unsigned long long d = (unsigned long long) pg_load_key(t + koff, kbytes) - (unsigned long long) dmin;
		const uint32_t e = (uint32_t) (hj_pack_value(t, bc) - vmin);
		if (atomicExch(&table[d], e) != 0xFFFFFFFFu) dup = true;
	}
	if (dup) atomicOr(flags, 1);
}

// 16-byte build tuples (8-byte key at word 0 or 2, 16-byte aligned): one
// vector load per tuple, four tuples in flight per thread.
__device__ __forceinline__ uint32_t hj_word4(const uint4& t, uint32_t i)
{
	return i == 0 ? t.x : i == 1 ? t.y : i == 2 ? t.z : t.w;
}

// The packed value's word positions in a 16-byte tuple as one word for the
// kernels of the device-side build: bits 0-1 the number of words (0..2),
// bits 2-3 and 4-5 the tuple words (a structure parameter indexed at run
// time would be copied to local memory).
static uint32_t hj_pack16_code(const HjBuildCols& bc)
{
	uint32_t code = 0, o = 0;
	for (int c = 0; c < bc.n; ++c)
		for (int j = 0; j < bc.words[c] && o < 2; ++j, ++o) code |= (uint32_t) ((bc.roff[c] + j) & 3) << (2 + 2 * o);
	return code | o;
}

__device__ __forceinline__ uint64_t hj_pack16(const uint4& t, uint32_t code)
{
	const uint32_t nw = code & 3;
	uint64_t v = 0;
	if (nw > 0) v = hj_word4(t, (code >> 2) & 3);
	if (nw > 1) v |= (uint64_t) hj_word4(t, (code >> 4) & 3) << 32;
	return v;
}

// (At most two words: packed values are 8 bytes or less. Built by shifts,
// not an indexed array, so nothing goes to local memory.)
__device__ __forceinline__ uint64_t hj_pack_value16(const uint4& t, const HjBuildCols& bc)
{
	uint64_t v = 0;
	uint32_t o = 0;
	for (int c = 0; c < bc.n; ++c)
		for (int j = 0; j < bc.words[c]; ++j, ++o)
			if (o < 2) v |= (uint64_t) hj_word4(t, bc.roff[c] + j) << (32 * o);
	return v;
}

__global__ void k_key_minmax16(const uint4* __restrict__ R, uint64_t n, uint32_t kw, HjBuildCols bc,
		unsigned long long* __restrict__ mm)
{
	unsigned long long lo = ~0ull, hi = 0, vlo = ~0ull, vhi = 0;
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	for (uint64_t i0 = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
		uint4 t[4];
		#pragma unroll
		for (int u = 0; u < 4; ++u) if (i0 + u * stride < n) t[u] = __ldg(R + i0 + u * stride);
		#pragma unroll
		for (int u = 0; u < 4; ++u) {
			if (i0 + u * stride >= n) break;
			const unsigned long long key = ((unsigned long long) hj_word4(t[u], kw + 1) << 32) | hj_word4(t[u], kw);
			const unsigned long long k = key ^ (1ull << 63);
			const unsigned long long v = hj_pack_value16(t[u], bc);
			lo = k < lo ? k : lo; hi = k > hi ? k : hi;
			vlo = v < vlo ? v : vlo; vhi = v > vhi ? v : vhi;
		}
	}
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		unsigned long long a = __shfl_down_sync(0xffffffffu, lo, o), b = __shfl_down_sync(0xffffffffu, hi, o);
		unsigned long long c = __shfl_down_sync(0xffffffffu, vlo, o), d = __shfl_down_sync(0xffffffffu, vhi, o);
		lo = a < lo ? a : lo; hi = b > hi ? b : hi;
		vlo = c < vlo ? c : vlo; vhi = d > vhi ? d : vhi;
	}
	if ((threadIdx.x & 31) == 0) {
		atomicMin(&mm[0], lo); atomicMax(&mm[1], hi);
		atomicMin(&mm[2], vlo); atomicMax(&mm[3], vhi);
	}
}

// Narrow dense table from 16-byte tuples with plain stores; duplicates are
// found afterwards by counting present entries (k_dense32_count < n).
__global__ void k_dense32_store16(const uint4* __restrict__ R, uint64_t n, uint32_t kw, HjBuildCols bc,
		long long dmin, unsigned long long vmin, uint32_t* __restrict__ table)
{
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	for (uint64_t i0 = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i0 < n; i0 += 4 * stride) {
		uint4 t[4];
		#pragma unroll
		for (int u = 0; u < 4; ++u) if (i0 + u * stride < n) t[u] = __ldg(R + i0 + u * stride);
		#pragma unroll
		for (int u = 0; u < 4; ++u) {
			if (i0 + u * stride >= n) break;
			const unsigned long long key = ((unsigned long long) hj_word4(t[u], kw + 1) << 32) | hj_word4(t[u], kw);
			table[key - (unsigned long long) dmin] = (uint32_t) (hj_pack_value16(t[u], bc) - vmin);
		}
	}
}

// Present entries (not all ones) of a narrow dense table of `range` entries.
__global__ void k_dense32_count(const uint32_t* __restrict__ table, uint64_t range, unsigned long long* __restrict__ cnt)
{
	unsigned long long c = 0;
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	const uint64_t n4 = range / 4;
	const uint4* t4 = reinterpret_cast<const uint4*>(table);
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n4; i += stride) {
		const uint4 v = t4[i];
		c += (v.x != 0xFFFFFFFFu) + (v.y != 0xFFFFFFFFu) + (v.z != 0xFFFFFFFFu) + (v.w != 0xFFFFFFFFu);
	}
	for (uint64_t i = 4 * n4 + blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < range; i += stride)
		c += table[i] != 0xFFFFFFFFu;
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
	if ((threadIdx.x & 31) == 0 && c) atomicAdd(cnt, c);
}

// ---------------------------------------------------------------------------
// Narrow dense build of 16-byte tuples without host round trips. The layout
// is chosen from a sample and checked afterwards: a key outside the window, a
// value outside the entry range or fewer present entries than tuples (a
// repeated key) marks the header bad, and the table's first use rebuilds it
// exactly. Four launches: sample, fill, store, count.
// ---------------------------------------------------------------------------
#define HJ_SPEC_SAMPLE 4096
#define HJ_SPEC_MIN_TUPLES 65536

__device__ __forceinline__ void hj_minmax4(unsigned long long& lo, unsigned long long& hi, unsigned long long& vlo,
		unsigned long long& vhi)
{
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		unsigned long long a = __shfl_down_sync(0xffffffffu, lo, o), b = __shfl_down_sync(0xffffffffu, hi, o);
		unsigned long long c = __shfl_down_sync(0xffffffffu, vlo, o), d = __shfl_down_sync(0xffffffffu, vhi, o);
		lo = a < lo ? a : lo; hi = b > hi ? b : hi;
		vlo = c < vlo ? c : vlo; vhi = d > vhi ? d : vhi;
	}
}

// One CTA of 1024 threads: key and value ranges of HJ_SPEC_SAMPLE evenly
// spaced build tuples (all of them when fewer) set the window: the sampled key
// span widened by a sixteenth of itself plus 1024 keys on each side (exact
// when every tuple was sampled), and the value base: 0 when the sampled
// values leave room for it, else centred on them. `cap` = entries allocated.
__global__ void __launch_bounds__(1024) k_dense_prep16(const uint4* __restrict__ R, uint64_t n, uint32_t kw,
		uint32_t pk, uint64_t cap, HjDenseHdr* __restrict__ hdr)
{
	__shared__ unsigned long long red[4][32];
	const uint64_t m = n < HJ_SPEC_SAMPLE ? n : HJ_SPEC_SAMPLE;
	const uint64_t q = n / m, r = n % m;
	unsigned long long lo = ~0ull, hi = 0, vlo = ~0ull, vhi = 0;
	for (uint64_t t = threadIdx.x; t < m; t += blockDim.x) {
		const uint64_t i = t * q + (t * r) / m;      // < n: t < m, t*r < 2^24
		const uint4 v = __ldg(R + i);
		const unsigned long long k = (((unsigned long long) hj_word4(v, kw + 1) << 32) | hj_word4(v, kw)) ^ (1ull << 63);
		const unsigned long long p = hj_pack16(v, pk);
		lo = k < lo ? k : lo; hi = k > hi ? k : hi;
		vlo = p < vlo ? p : vlo; vhi = p > vhi ? p : vhi;
	}
	hj_minmax4(lo, hi, vlo, vhi);
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	if (lane == 0) { red[0][warp] = lo; red[1][warp] = hi; red[2][warp] = vlo; red[3][warp] = vhi; }
	__syncthreads();
	if (warp != 0) return;
	const int nw = blockDim.x >> 5;
	lo = lane < nw ? red[0][lane] : ~0ull; hi = lane < nw ? red[1][lane] : 0;
	vlo = lane < nw ? red[2][lane] : ~0ull; vhi = lane < nw ? red[3][lane] : 0;
	hj_minmax4(lo, hi, vlo, vhi);
	if (lane != 0) return;
	HjDenseHdr h;
	h.n = n; h.present = 0; h.kmin = ~0ull; h.kmax = 0; h.vlo = ~0ull; h.vhi = 0; h.flags = 0; h.pad = 0;
	unsigned long long wlo = lo, whi = hi;
	if (m != n) {
		const unsigned long long d = (hi - lo) / 16 + 1024;
		wlo = lo >= d ? lo - d : 0;
		whi = hi <= ~0ull - d ? hi + d : ~0ull;
	}
	h.dmin = (long long) (wlo ^ (1ull << 63));
	h.drange = whi - wlo < cap ? whi - wlo + 1 : 0;
	const unsigned long long vspan = vhi - vlo;
	h.vmin = 0;
	if (h.drange == 0 || vspan >= 0xFFFFFFFEull) {
		h.flags = 4;
		h.drange = 0;
	} else {
		const unsigned long long slack = m == n ? 0 : (0xFFFFFFFEull - vspan) / 2;
		h.vmin = vlo <= slack ? 0 : vlo - slack;
	}
	*hdr = h;
}

// All ones over the window's entries (nothing when the sample ruled it out).
__global__ void k_dense_fill16(uint32_t* __restrict__ table, const HjDenseHdr* __restrict__ hdr)
{
	const unsigned long long range = hdr->drange;
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	const uint64_t n4 = range / 4;
	uint4* t4 = reinterpret_cast<uint4*>(table);
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n4; i += stride)
		t4[i] = make_uint4(~0u, ~0u, ~0u, ~0u);
	for (uint64_t i = 4 * n4 + blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < range; i += stride)
		table[i] = ~0u;
}

// Store pass: entry key - dmin = value - vmin, plain stores kept in L2
// (evict-last measured fastest for the scattered 4-byte stores), eight build
// tuples in flight per thread read evict-first; flags keys outside the window
// and values outside the entry range.
__global__ void __launch_bounds__(256) k_dense32_spec16(const uint4* __restrict__ R, uint64_t n, uint32_t kw,
		uint32_t pk, uint32_t* __restrict__ table, HjDenseHdr* __restrict__ hdr)
{
	if (hdr->flags) return;
	const unsigned long long dmin = (unsigned long long) hdr->dmin, range = hdr->drange, vmin = hdr->vmin;
	const uint64_t keep = pg_policy_evict_last(), stream = pg_policy_evict_first();
	int bad = 0;
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	for (uint64_t i0 = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i0 < n; i0 += 8 * stride) {
		uint4 t[8];
		#pragma unroll
		for (int u = 0; u < 8; ++u)
			if (i0 + u * stride < n) t[u] = pg_ld_hint16(R + i0 + u * stride, stream);
		#pragma unroll
		for (int u = 0; u < 8; ++u) {
			if (i0 + u * stride >= n) break;
			const unsigned long long key = ((unsigned long long) hj_word4(t[u], kw + 1) << 32) | hj_word4(t[u], kw);
			const unsigned long long d = key - dmin, e = hj_pack16(t[u], pk) - vmin;
			if (d >= range) bad |= 1;
			else if (e >= 0xFFFFFFFFull) bad |= 2;
			else asm volatile("st.global.L2::cache_hint.u32 [%0], %1, %2;"
					:: "l"(table + d), "r"((uint32_t) e), "l"(keep) : "memory");
		}
	}
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) bad |= __shfl_down_sync(0xffffffffu, bad, o);
	if ((threadIdx.x & 31) == 0 && bad) atomicOr(&hdr->flags, bad);
}

// Count pass: present entries of the window into hdr->present (equal to n
// exactly when no key repeated), and the exact key and value ranges from the
// first and last present entries and the smallest and largest entry. Each
// thread reads its 16-byte words four at a time (four loads in flight: one at
// a time the pass waited on DRAM latency), and since its words come in
// increasing order, its first and last present index need no compares.
__global__ void k_dense32_count_spec(const uint32_t* __restrict__ table, HjDenseHdr* __restrict__ hdr)
{
	if (hdr->flags) return;
	const unsigned long long range = hdr->drange;
	unsigned long long c = 0, dlo = ~0ull, dhi = 0;
	uint32_t elo = 0xFFFFFFFFu, ehi = 0;
	auto see = [&](uint32_t e, unsigned long long d) {
		if (e == 0xFFFFFFFFu) return;
		++c;
		if (dlo == ~0ull) dlo = d;
		dhi = d;
		elo = e < elo ? e : elo;
		ehi = e > ehi ? e : ehi;
	};
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	const uint64_t n4 = range / 4;
	const uint4* t4 = reinterpret_cast<const uint4*>(table);
	uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x;
	for (; i + 3 * stride < n4; i += 4 * stride) {
		uint4 v[4];
		#pragma unroll
		for (int j = 0; j < 4; ++j) v[j] = t4[i + j * stride];
		#pragma unroll
		for (int j = 0; j < 4; ++j) {
			const unsigned long long d = 4 * (i + j * stride);
			see(v[j].x, d); see(v[j].y, d + 1); see(v[j].z, d + 2); see(v[j].w, d + 3);
		}
	}
	for (; i < n4; i += stride) {
		const uint4 v = t4[i];
		see(v.x, 4 * i); see(v.y, 4 * i + 1); see(v.z, 4 * i + 2); see(v.w, 4 * i + 3);
	}
	for (uint64_t j = 4 * n4 + blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; j < range; j += stride)
		see(table[j], j);
	unsigned long long vlo = c ? elo : ~0ull, vhi = ehi;
	hj_minmax4(dlo, dhi, vlo, vhi);
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
	// One set of header atomics per CTA, not per warp: the five words share
	// one L2 line, where thousands of warps' atomics queued up.
	__shared__ unsigned long long red[5][8];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	if (lane == 0) { red[0][warp] = c; red[1][warp] = dlo; red[2][warp] = dhi; red[3][warp] = vlo; red[4][warp] = vhi; }
	__syncthreads();
	if (threadIdx.x == 0) {
		for (int w = 1; w < (int) (blockDim.x >> 5); ++w) {
			c += red[0][w];
			dlo = red[1][w] < dlo ? red[1][w] : dlo; dhi = red[2][w] > dhi ? red[2][w] : dhi;
			vlo = red[3][w] < vlo ? red[3][w] : vlo; vhi = red[4][w] > vhi ? red[4][w] : vhi;
		}
		if (c) {
			const unsigned long long dmin = (unsigned long long) hdr->dmin, vmin = hdr->vmin;
			atomicAdd(&hdr->present, c);
			atomicMin(&hdr->kmin, (dmin + dlo) ^ (1ull << 63)); atomicMax(&hdr->kmax, (dmin + dhi) ^ (1ull << 63));
			atomicMin(&hdr->vlo, vmin + vlo); atomicMax(&hdr->vhi, vmin + vhi);
		}
	}
}

// Entries of a settled table re-based from the sample's value base to the
// exact smallest value, into a new array: present entries drop by `shift`.
__global__ void k_dense32_rebase(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, uint64_t range,
		uint32_t shift)
{
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < range; i += (uint64_t) gridDim.x * blockDim.x) {
		const uint32_t e = src[i];
		dst[i] = e != 0xFFFFFFFFu ? e - shift : e;
	}
}

// Probe kernels given a speculative table read its window here; false: the
// build's checks failed, the kernel does nothing and the host rebuilds.
__device__ __forceinline__ bool hj_spec_resolve(HjProbeTable& tb)
{
	if (!tb.hdr) return true;
	const HjDenseHdr* h = tb.hdr;
	if (h->flags != 0 || h->present != h->n) return false;
	tb.dmin = h->dmin;
	tb.drange = h->drange;
	tb.vmin = h->vmin;
	return true;
}

// Dense table: presence bit and value at key - dmin. A bit found already set
// means a duplicate key; the host then builds the hashed table instead.
__global__ void k_dense_build(const char* __restrict__ R, uint64_t n, uint32_t W, uint32_t koff,
		uint32_t kbytes, HjBuildCols bc, bool inline_val, long long dmin,
		unsigned long long* __restrict__ dval, uint32_t* __restrict__ dbits, int* __restrict__ flags)
{
	bool dup = false;
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
			i += (uint64_t) gridDim.x * blockDim.x) {
		const char* t = R + i * W;
		const unsigned long long d = (unsigned long long) pg_load_key(t + koff, kbytes) - (unsigned long long) dmin;
		uint64_t v = i;
		if (inline_val) {
			uint32_t w[2] = {0, 0};
			int o = 0;
			for (int c = 0; c < bc.n; ++c)
				for (int j = 0; j < bc.words[c]; ++j) w[o++] = hj_word(t, bc.roff[c] + j);
			v = ((uint64_t) w[1] << 32) | w[0];
		}
		const uint32_t bit = 1u << (d & 31);
		if (atomicOr(&dbits[d >> 5], bit) & bit) dup = true;
		dval[d] = v;
	}
	if (dup) atomicOr(flags, 1);
}

// Value of output word `w` for a match: from the probe tuple or from the build
// side (packed value, or the build tuple when values are row indices).
__device__ __forceinline__ uint32_t hj_out_word(const HjCols& pc, int c, int j, const char* ptup,
		uint64_t val, bool inline_val, const char* R, uint32_t wR)
{
	if (pc.side[c]) return hj_word(ptup, pc.src[c] + j);
	if (inline_val) {
		uint32_t idx = pc.src[c] + j;
		return idx == 0 ? (uint32_t) val : (uint32_t) (val >> 32);
	}
	return hj_word(R + val * wR, pc.src[c] + j);
}

// ---------------------------------------------------------------------------
// Unique-key probe: one pass, tile-ordered output, one atomicAdd per tile.
// FAST16: probe tuples are 16 bytes and output rows 16 bytes (4 words).
// ---------------------------------------------------------------------------
// Single lookup in a unique-key table (hashed or dense). Returns whether key
// k is present and its value.
__device__ __forceinline__ bool hj_lookup_unique(const HjProbeTable& tb, bool dense, int64_t k, uint64_t& val)
{
	if (dense) {
		const unsigned long long d = (unsigned long long) k - (unsigned long long) tb.dmin;
		if (d >= tb.drange) return false;
		if (tb.dense32) {
			const uint32_t e = tb.dense32[d];
			val = tb.vmin + e;
			return e != 0xFFFFFFFFu;
		}
		if (!((tb.dense_bits[d >> 5] >> (d & 31)) & 1)) return false;
		val = tb.dense_val[d];
		return true;
	}
	if (k == PG_EMPTY_KEY) {
		if (!tb.nside) return false;
		val = tb.side[0];
		return true;
	}
	const uint64_t mask = (1ull << tb.log2cap) - 1;
	uint64_t s = hj_slot0(k, tb.log2cap);
	for (uint64_t probe = 0; probe <= mask; ++probe) {
		const uint4 v = pg_ld_table16(tb.slots + 2 * s);
		const int64_t sk = (int64_t) (((uint64_t) v.y << 32) | v.x);
		if (sk == k) { val = ((uint64_t) v.w << 32) | v.z; return true; }
		if (sk == PG_EMPTY_KEY) return false;
		s = (s + 1) & mask;
	}
	return false;
}

template <bool MATERIALIZE, bool FAST16>
__global__ void __launch_bounds__(HJ_THREADS)
k_probe_unique(const char* __restrict__ S, uint64_t n, uint32_t W, uint32_t koff, uint32_t kbytes,
		const HjProbeTable tb, bool dense,
		HjCols pc, char* __restrict__ out, uint64_t out_cap,
		unsigned long long* __restrict__ cursor, unsigned long long* __restrict__ agg,
		int sum_col, int* __restrict__ status)
{
	__shared__ uint32_t wcnt[HJ_ITEMS][HJ_THREADS / 32];
	__shared__ unsigned long long tile_base;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const uint64_t ntiles = pg_div_up(n, HJ_TILE);
	unsigned long long cnt_acc = 0, sum_acc = 0;

	for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
		const uint64_t base = tile * HJ_TILE;
		uint4 tup[HJ_ITEMS];
		int64_t key[HJ_ITEMS];
		uint64_t val[HJ_ITEMS];
		bool hit[HJ_ITEMS];
		// Load probe tuples (streaming) and their first table slot (L2-resident).
		#pragma unroll
		for (int j = 0; j < HJ_ITEMS; ++j) {
			uint64_t r = base + (uint64_t) j * HJ_THREADS + tid;
			hit[j] = false;
			key[j] = 0;
			if (r < n) {
				if (FAST16) {
					tup[j] = pg_ld_stream16(S + r * 16);
					key[j] = (int64_t) (((uint64_t) tup[j].y << 32) | tup[j].x);
					if (koff == 8) key[j] = (int64_t) (((uint64_t) tup[j].w << 32) | tup[j].z);
				} else {
					key[j] = pg_load_key(S + r * W + koff, kbytes);
				}
			}
		}
		#pragma unroll
		for (int j = 0; j < HJ_ITEMS; ++j) {
			uint64_t r = base + (uint64_t) j * HJ_THREADS + tid;
			if (r < n) hit[j] = hj_lookup_unique(tb, dense, key[j], val[j]);
		}
		if (MATERIALIZE) {
			// Tile-order ranks: item-major, then warp, then lane.
			uint32_t ball[HJ_ITEMS];
			#pragma unroll
			for (int j = 0; j < HJ_ITEMS; ++j) {
				ball[j] = __ballot_sync(0xffffffffu, hit[j]);
				if (lane == 0) wcnt[j][warp] = __popc(ball[j]);
			}
			__syncthreads();
			if (tid == 0) {
				uint32_t run = 0;
				for (int j = 0; j < HJ_ITEMS; ++j)
					for (int w = 0; w < HJ_THREADS / 32; ++w) { uint32_t c = wcnt[j][w]; wcnt[j][w] = run; run += c; }
				tile_base = atomicAdd(cursor, (unsigned long long) run);
			}
			__syncthreads();
			const unsigned long long tb = tile_base;
			#pragma unroll
			for (int j = 0; j < HJ_ITEMS; ++j) {
				if (!hit[j]) continue;
				uint64_t pos = tb + wcnt[j][warp] + __popc(ball[j] & ((1u << lane) - 1));
				if (pos >= out_cap) continue;
				if (FAST16) {
					uint32_t w4[4];
					int o = 0;
					for (int c = 0; c < pc.n; ++c)
						for (int q = 0; q < pc.words[c]; ++q) {
							uint32_t src = pc.src[c] + q, x;
							if (pc.side[c]) x = src == 0 ? tup[j].x : src == 1 ? tup[j].y : src == 2 ? tup[j].z : tup[j].w;
							else x = src == 0 ? (uint32_t) val[j] : (uint32_t) (val[j] >> 32);
							w4[o++] = x;
						}
					pg_st_stream16(out + pos * 16, make_uint4(w4[0], w4[1], w4[2], w4[3]));
				} else {
					uint32_t* o = reinterpret_cast<uint32_t*>(out + pos * (uint64_t) pc.ow_words * 4);
					const char* pt = S + (base + (uint64_t) j * HJ_THREADS + tid) * W;
					int wo = 0;
					for (int c = 0; c < pc.n; ++c)
						for (int q = 0; q < pc.words[c]; ++q)
							o[wo++] = hj_out_word(pc, c, q, pt, val[j], true, nullptr, 0);
				}
			}
			__syncthreads();
		} else {
			#pragma unroll
			for (int j = 0; j < HJ_ITEMS; ++j) {
				if (!hit[j]) continue;
				cnt_acc++;
				if (sum_col >= 0) {
					const char* pt = S + (base + (uint64_t) j * HJ_THREADS + tid) * W;
					uint32_t lo = hj_out_word(pc, sum_col, 0, pt, val[j], true, nullptr, 0);
					if (pc.words[sum_col] == 2) {
						uint32_t hi = hj_out_word(pc, sum_col, 1, pt, val[j], true, nullptr, 0);
						sum_acc += ((unsigned long long) hi << 32) | lo;
					} else {
						sum_acc += (unsigned long long) (long long) (int32_t) lo;
					}
				}
			}
		}
	}
	if (!MATERIALIZE) {
		#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			cnt_acc += __shfl_down_sync(0xffffffffu, cnt_acc, o);
			sum_acc += __shfl_down_sync(0xffffffffu, sum_acc, o);
		}
		if (lane == 0) { atomicAdd(&agg[0], cnt_acc); atomicAdd(&agg[1], sum_acc); }
	}
}

// ---------------------------------------------------------------------------
// Unique-key probe of 16-byte tuples, Blackwell path. Per CTA, persistent over
// tiles of 1024 probe tuples:
//   * tiles arrive in shared memory by bulk copy (cp.async.bulk + mbarrier,
//     L2 evict-first), the next tile prefetched while the current one is
//     probed;
//   * each thread resolves 4 keys. Hashed tables: every key's first 32-byte
//     bucket (two slots) is fetched with one 256-bit evict-last load, all
//     issued before any is inspected, and keys needing a further bucket
//     advance together in rounds. Dense tables: one bitmap word and one
//     8-byte value per key, both issued at once;
//   * matches are ranked in tile order (warp ballots + per-warp prefix),
//     assembled as output rows in shared memory, and written with one bulk
//     store per tile (evict-first) into a range reserved by a single
//     atomicAdd that only the issuing thread waits on.
// ---------------------------------------------------------------------------
#define HJT_TILE 1024
#define HJT_THREADS 256
#define HJT_ITEMS (HJT_TILE / HJT_THREADS)
#define HJT_WARPS (HJT_THREADS / 32)

__device__ __forceinline__ uint32_t hj_pick(const uint4& t, uint64_t v, uint32_t i)
{
	uint32_t r = t.x;
	r = i == 1 ? t.y : r;
	r = i == 2 ? t.z : r;
	r = i == 3 ? t.w : r;
	r = i == 4 ? (uint32_t) v : r;
	r = i == 5 ? (uint32_t) (v >> 32) : r;
	return r;
}

template <bool MATERIALIZE, int MODE>
__global__ void __launch_bounds__(HJT_THREADS, 3)
k_probe16_tma(const char* __restrict__ S, uint64_t n, uint32_t koff, const HjProbeTable tb,
		uint32_t wsel, uint32_t sum_w0, uint32_t sum_words, char* __restrict__ out, uint64_t out_cap,
		unsigned long long* __restrict__ cursor, unsigned long long* __restrict__ agg,
		int sum_col, int* __restrict__ status)
{
	extern __shared__ __align__(128) unsigned char sm[];
	uint4* const tin0 = reinterpret_cast<uint4*>(sm);
	uint4* const tout = reinterpret_cast<uint4*>(sm + 2 * HJT_TILE * 16);
	__shared__ __align__(8) uint64_t bar[2];
	__shared__ uint32_t wsum[HJT_WARPS];
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const uint64_t mask = (1ull << tb.log2cap) - 1;
	const uint64_t ntiles = pg_div_up(n, HJT_TILE);
	const uint64_t keep = pg_policy_evict_last();
	const uint64_t stream = pg_policy_evict_first();
	unsigned long long cnt_acc = 0, sum_acc = 0;
	// Output word i is source word (wsel >> 4i) & 15 of (probe tuple words
	// 0-3, packed build value words 4-5).
	const uint32_t w0 = wsel & 15, w1 = (wsel >> 4) & 15, w2 = (wsel >> 8) & 15, w3 = (wsel >> 12) & 15;
	if (tid == 0) { pg_mbar_init(&bar[0], 1); pg_mbar_init(&bar[1], 1); pg_fence_mbar_init(); }
	__syncthreads();
	uint64_t tile = blockIdx.x;
	if (tile >= ntiles) return;
	auto issue = [&](uint64_t t, int b) {
		const uint32_t rows = (uint32_t) pg_min64(HJT_TILE, n - t * HJT_TILE);
		pg_mbar_expect_tx(&bar[b], rows * 16);
		pg_bulk_g2s_hint(tin0 + b * HJT_TILE, S + t * (uint64_t) HJT_TILE * 16, rows * 16, &bar[b], stream);
	};
	if (tid == 0) issue(tile, 0);
	uint32_t phases = 0;     // bit b: parity expected next on bar[b]
	const uint32_t spin = pg_spin_knob(status);
	for (int it = 0; tile < ntiles; tile += gridDim.x, ++it) {
		const int b = it & 1;
		const uint4* const tp = tin0 + b * HJT_TILE;
		const uint64_t base = tile * HJT_TILE;
		const uint32_t rows = (uint32_t) pg_min64(HJT_TILE, n - base);
		// A wait past the context's limit records PG_ERR_TIMEOUT and drains
		// the copy; if even that gives up, the tile's contents are
		// unspecified, every later access stays in bounds and the host sees
		// the status.
		pg_mbar_wait_timed(&bar[b], (phases >> b) & 1, spin, status);
		phases ^= 1u << b;
		// Prefetch the next tile into the other buffer; its previous contents
		// were last read before the final barrier of the previous tile.
		if (tid == 0 && tile + gridDim.x < ntiles) issue(tile + gridDim.x, b ^ 1);

		int64_t key[HJT_ITEMS];
		uint64_t val[HJT_ITEMS];
		bool hit[HJT_ITEMS];
		if (MODE != 0) {
			uint32_t bits[HJT_ITEMS];
			#pragma unroll
			for (int j = 0; j < HJT_ITEMS; ++j) {
				const uint32_t p = j * HJT_THREADS + tid;
				hit[j] = false; val[j] = 0; bits[j] = 0;
				if (p < rows) {
					const uint4 t = tp[p];
					key[j] = koff == 0 ? (int64_t) (((uint64_t) t.y << 32) | t.x) : (int64_t) (((uint64_t) t.w << 32) | t.z);
					const unsigned long long d = (unsigned long long) key[j] - (unsigned long long) tb.dmin;
					if (d < tb.drange) {
						if (MODE == 2) {
							uint32_t e;
							asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;"
									: "=r"(e) : "l"(tb.dense32 + d), "l"(keep));
							bits[j] = e != 0xFFFFFFFFu;
							val[j] = tb.vmin + e;
						} else {
							bits[j] = __ldg(tb.dense_bits + (d >> 5)) >> (d & 31);
							asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u64 %0, [%1], %2;"
									: "=l"(val[j]) : "l"(tb.dense_val + d), "l"(keep));
						}
						hit[j] = true;
					}
				}
			}
			#pragma unroll
			for (int j = 0; j < HJT_ITEMS; ++j) hit[j] = hit[j] && (bits[j] & 1);
		} else {
			uint64_t slot[HJT_ITEMS];
			bool open[HJT_ITEMS];
			#pragma unroll
			for (int j = 0; j < HJT_ITEMS; ++j) {
				const uint32_t p = j * HJT_THREADS + tid;
				hit[j] = false; open[j] = false; val[j] = 0;
				key[j] = 0;
				if (p < rows) {
					const uint4 t = tp[p];
					key[j] = koff == 0 ? (int64_t) (((uint64_t) t.y << 32) | t.x) : (int64_t) (((uint64_t) t.w << 32) | t.z);
					if (key[j] == PG_EMPTY_KEY) { if (tb.nside) { hit[j] = true; val[j] = tb.side[0]; } }
					else { open[j] = true; slot[j] = hj_slot0(key[j], tb.log2cap); }
				}
			}
			// Rounds of bucket loads: all open keys issue, then all inspect.
			for (uint32_t round = 0; round <= (mask >> 1); ++round) {
				pg_u64x4 bk[HJT_ITEMS];
				bool any = false;
				#pragma unroll
				for (int j = 0; j < HJT_ITEMS; ++j)
					if (open[j]) { bk[j] = pg_ld_bucket32(tb.slots + 2 * slot[j], keep); any = true; }
				if (!any) break;
				#pragma unroll
				for (int j = 0; j < HJT_ITEMS; ++j) {
					if (!open[j]) continue;
					if ((long long) bk[j].a == key[j]) { hit[j] = true; val[j] = bk[j].b; open[j] = false; }
					else if (bk[j].a == (unsigned long long) PG_EMPTY_KEY) open[j] = false;
					else if ((long long) bk[j].c == key[j]) { hit[j] = true; val[j] = bk[j].d; open[j] = false; }
					else if (bk[j].c == (unsigned long long) PG_EMPTY_KEY) open[j] = false;
					else slot[j] = (slot[j] + 2) & mask;
				}
			}
		}
		if (MATERIALIZE) {
			// Row order in the tile: warp, then item, then lane.
			uint32_t ball[HJT_ITEMS], mine = 0;
			#pragma unroll
			for (int j = 0; j < HJT_ITEMS; ++j) { ball[j] = __ballot_sync(0xffffffffu, hit[j]); mine += __popc(ball[j]); }
			if (lane == 0) wsum[warp] = mine;
			// The output buffer is free once the previous tile's bulk store
			// has read it.
			if (tid == 0) pg_bulk_wait_read();
			__syncthreads();
			uint32_t pos = 0, total = 0;
			#pragma unroll
			for (int w = 0; w < HJT_WARPS; ++w) { uint32_t c = wsum[w]; pos += w < warp ? c : 0; total += c; }
			#pragma unroll
			for (int j = 0; j < HJT_ITEMS; ++j) {
				if (hit[j]) {
					const uint4 t = tp[j * HJT_THREADS + tid];
					tout[pos + __popc(ball[j] & ((1u << lane) - 1))] =
						make_uint4(hj_pick(t, val[j], w0), hj_pick(t, val[j], w1),
								hj_pick(t, val[j], w2), hj_pick(t, val[j], w3));
				}
				pos += __popc(ball[j]);
			}
			pg_fence_proxy_async_smem();
			__syncthreads();
			if (tid == 0 && total) {
				const unsigned long long at = atomicAdd(cursor, (unsigned long long) total);
				if (at + total <= out_cap) pg_bulk_s2g_hint(out + at * 16, tout, total * 16, stream);
			}
		} else {
			#pragma unroll
			for (int j = 0; j < HJT_ITEMS; ++j) {
				if (!hit[j]) continue;
				cnt_acc++;
				if (sum_col >= 0) {
					const uint4 t = tp[j * HJT_THREADS + tid];
					const uint32_t lo = hj_pick(t, val[j], (wsel >> (4 * sum_w0)) & 15);
					if (sum_words == 2)
						sum_acc += ((unsigned long long) hj_pick(t, val[j], (wsel >> (4 * sum_w0 + 4)) & 15) << 32) | lo;
					else sum_acc += (unsigned long long) (long long) (int32_t) lo;
				}
			}
			__syncthreads();   // tile buffer b is refilled by the next prefetch
		}
	}
	if (MATERIALIZE) {
		if (tid == 0) pg_bulk_wait_all();
	} else {
		#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			cnt_acc += __shfl_down_sync(0xffffffffu, cnt_acc, o);
			sum_acc += __shfl_down_sync(0xffffffffu, sum_acc, o);
		}
		if (lane == 0) { atomicAdd(&agg[0], cnt_acc); atomicAdd(&agg[1], sum_acc); }
	}
}

// ---------------------------------------------------------------------------
// Unique-key probe of tuples whose width is any multiple of 4 bytes (the
// 16-byte kernels below take only 16-byte tuples and rows), staged through
// shared memory. Per CTA, persistent over tiles of 256 * ITEMS probe tuples:
//   * a tile arrives by one bulk copy (cp.async.bulk + mbarrier, L2
//     evict-first) into one of three buffers, the copy of the CTA's next
//     tile issued before the current one is probed; the final tile's last
//     bytes past a multiple of 16 are loaded by the threads;
//   * keys are read from shared memory and looked up ITEMS per thread, all
//     table loads issued before any is used (hashed tables: rounds of 32-byte
//     bucket loads);
//   * a match records its tile row and build value at its rank in the tile
//     (warp, then item, then lane); the CTA then writes the output rows with
//     coalesced word stores, each word taken through an output-word map from
//     the staged probe tuple or the build value, into a range reserved by one
//     atomicAdd per tile.
// Three buffers let the next copy start at the top of an iteration: the one it
// overwrites was last read by the word stores of two tiles back, which every
// thread finished before the previous tile's first barrier.
// ---------------------------------------------------------------------------
#define HJG_THREADS 256
#define HJG_WARPS (HJG_THREADS / 32)
#define HJG_BUFS 3
#define HJG_MAX_OW 32        // output words (128-byte rows)
#define HJG_MAX_W 64         // probe tuple bytes staged (3 x 512-row buffers + row records: 2 CTAs per SM)

struct HjWordMap {
	uint8_t src[HJG_MAX_OW];  // output word o: probe tuple word src (< 64) or build value word src - 64
	uint32_t ow;              // output row words
	uint32_t uw;              // words per store: 2 when rows are a whole number of 8-byte units, else 1
	uint32_t sum_w0, sum_words;
};

__device__ __forceinline__ uint32_t hjg_word(const uint32_t* tw, uint64_t val, uint32_t src)
{
	return src < 64 ? tw[src] : (uint32_t) (val >> (32 * (src - 64)));
}

template <int MODE, int ITEMS>
__device__ __forceinline__ void hj_lookup_items(const HjProbeTable& tb, const int64_t (&key)[ITEMS],
		const bool (&valid)[ITEMS], bool (&hit)[ITEMS], uint64_t (&val)[ITEMS], uint64_t keep)
{
	if (MODE != 0) {
		uint32_t bits[ITEMS];
		#pragma unroll
		for (int j = 0; j < ITEMS; ++j) {
			hit[j] = false; val[j] = 0; bits[j] = 0;
			const unsigned long long d = (unsigned long long) key[j] - (unsigned long long) tb.dmin;
			if (valid[j] && d < tb.drange) {
				if (MODE == 2) {
					uint32_t e;
					asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;"
							: "=r"(e) : "l"(tb.dense32 + d), "l"(keep));
					bits[j] = e != 0xFFFFFFFFu;
					val[j] = tb.vmin + e;
				} else {
					bits[j] = __ldg(tb.dense_bits + (d >> 5)) >> (d & 31);
					asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u64 %0, [%1], %2;"
							: "=l"(val[j]) : "l"(tb.dense_val + d), "l"(keep));
				}
				hit[j] = true;
			}
		}
		#pragma unroll
		for (int j = 0; j < ITEMS; ++j) hit[j] = hit[j] && (bits[j] & 1);
	} else {
		const uint64_t mask = (1ull << tb.log2cap) - 1;
		uint64_t slot[ITEMS];
		bool open[ITEMS];
		#pragma unroll
		for (int j = 0; j < ITEMS; ++j) {
			hit[j] = false; open[j] = false; val[j] = 0; slot[j] = 0;
			if (!valid[j]) continue;
			if (key[j] == PG_EMPTY_KEY) { if (tb.nside) { hit[j] = true; val[j] = tb.side[0]; } }
			else { open[j] = true; slot[j] = hj_slot0(key[j], tb.log2cap); }
		}
		for (uint32_t round = 0; round <= (mask >> 1); ++round) {
			pg_u64x4 bk[ITEMS];
			bool any = false;
			#pragma unroll
			for (int j = 0; j < ITEMS; ++j)
				if (open[j]) { bk[j] = pg_ld_bucket32(tb.slots + 2 * slot[j], keep); any = true; }
			if (!any) break;
			#pragma unroll
			for (int j = 0; j < ITEMS; ++j) {
				if (!open[j]) continue;
				if ((long long) bk[j].a == key[j]) { hit[j] = true; val[j] = bk[j].b; open[j] = false; }
				else if (bk[j].a == (unsigned long long) PG_EMPTY_KEY) open[j] = false;
				else if ((long long) bk[j].c == key[j]) { hit[j] = true; val[j] = bk[j].d; open[j] = false; }
				else if (bk[j].c == (unsigned long long) PG_EMPTY_KEY) open[j] = false;
				else slot[j] = (slot[j] + 2) & mask;
			}
		}
	}
}

// Copy of tile t (T tuples of W bytes) into buffer b: the largest multiple of
// 16 bytes by one bulk copy completing on bar[b].
__device__ __forceinline__ void hjg_issue(const char* S, uint64_t n, uint32_t W, uint32_t T, uint64_t t,
		unsigned char* tin0, uint64_t* bar, int b, uint64_t pol)
{
	const uint32_t bytes = (uint32_t) pg_min64(T, n - t * T) * W;
	const uint32_t bulk = bytes & ~15u;
	pg_mbar_expect_tx(&bar[b], bulk);
	if (bulk) pg_bulk_g2s_hint(tin0 + (size_t) b * T * W, S + t * (uint64_t) T * W, bulk, &bar[b], pol);
}

// Table loads of one tile's ITEMS keys per thread, issued and not yet used:
// dense tables the 4-byte entry (narrow) or the bitmap word and 8-byte value
// (wide); hashed tables the first 32-byte bucket.
template <int MODE, int ITEMS>
struct HjPending {
	uint32_t e[ITEMS];
	uint64_t v[ITEMS];
	pg_u64x4 bk[ITEMS];
	uint64_t slot[ITEMS];
	bool in[ITEMS];
};

template <int MODE, int ITEMS>
__device__ __forceinline__ void hj_issue_items(const HjProbeTable& tb, const int64_t (&key)[ITEMS],
		const bool (&valid)[ITEMS], HjPending<MODE, ITEMS>& pd, uint64_t keep)
{
	#pragma unroll
	for (int j = 0; j < ITEMS; ++j) {
		pd.in[j] = false;
		if (MODE != 0) {
			const unsigned long long d = (unsigned long long) key[j] - (unsigned long long) tb.dmin;
			pd.e[j] = 0xFFFFFFFFu;
			if (!valid[j] || d >= tb.drange) continue;
			pd.in[j] = true;
			if (MODE == 2) {
				asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;"
						: "=r"(pd.e[j]) : "l"(tb.dense32 + d), "l"(keep));
			} else {
				pd.e[j] = __ldg(tb.dense_bits + (d >> 5)) >> (d & 31);
				asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u64 %0, [%1], %2;"
						: "=l"(pd.v[j]) : "l"(tb.dense_val + d), "l"(keep));
			}
		} else {
			if (!valid[j] || key[j] == PG_EMPTY_KEY) continue;
			pd.in[j] = true;
			pd.slot[j] = hj_slot0(key[j], tb.log2cap);
			pd.bk[j] = pg_ld_bucket32(tb.slots + 2 * pd.slot[j], keep);
		}
	}
}

// Uses the loads hj_issue_items started: hit and value per key (hashed keys
// that need further buckets probe on, in rounds, here).
template <int MODE, int ITEMS>
__device__ __forceinline__ void hj_resolve_items(const HjProbeTable& tb, const int64_t (&key)[ITEMS],
		const bool (&valid)[ITEMS], HjPending<MODE, ITEMS>& pd, bool (&hit)[ITEMS], uint64_t (&val)[ITEMS],
		uint64_t keep)
{
	if (MODE != 0) {
		#pragma unroll
		for (int j = 0; j < ITEMS; ++j) {
			if (MODE == 2) { hit[j] = pd.in[j] && pd.e[j] != 0xFFFFFFFFu; val[j] = tb.vmin + pd.e[j]; }
			else { hit[j] = pd.in[j] && (pd.e[j] & 1); val[j] = pd.in[j] ? pd.v[j] : 0; }
		}
		return;
	}
	const uint64_t mask = (1ull << tb.log2cap) - 1;
	#pragma unroll
	for (int j = 0; j < ITEMS; ++j) {
		hit[j] = false; val[j] = 0;
		if (valid[j] && key[j] == PG_EMPTY_KEY && tb.nside) { hit[j] = true; val[j] = tb.side[0]; }
	}
	for (uint32_t round = 0; ; ++round) {
		bool any = false;
		#pragma unroll
		for (int j = 0; j < ITEMS; ++j) {
			if (!pd.in[j]) continue;
			const pg_u64x4 b = pd.bk[j];
			if ((long long) b.a == key[j]) { hit[j] = true; val[j] = b.b; pd.in[j] = false; }
			else if (b.a == (unsigned long long) PG_EMPTY_KEY) pd.in[j] = false;
			else if ((long long) b.c == key[j]) { hit[j] = true; val[j] = b.d; pd.in[j] = false; }
			else if (b.c == (unsigned long long) PG_EMPTY_KEY) pd.in[j] = false;
			else if (round >= (mask >> 1)) pd.in[j] = false;     // every bucket seen
			else pd.slot[j] = (pd.slot[j] + 2) & mask;
		}
		#pragma unroll
		for (int j = 0; j < ITEMS; ++j)
			if (pd.in[j]) { pd.bk[j] = pg_ld_bucket32(tb.slots + 2 * pd.slot[j], keep); any = true; }
		if (!any) break;
	}
}

// Waits for the tile in buffer b (bounded: a wait that gives up leaves the
// tile's contents unspecified, every access stays in bounds and the host sees
// the status); the final tile's bytes past a multiple of 16 are loaded here.
__device__ __forceinline__ void hjg_arrive(const char* S, uint64_t base, uint32_t rows, uint32_t W,
		unsigned char* tp, uint64_t* bar, int b, uint32_t& phases, int* status)
{
	pg_mbar_wait_timed(&bar[b], (phases >> b) & 1, pg_spin_knob(status), status);
	phases ^= 1u << b;
	const uint32_t bytes = rows * W, bulk = bytes & ~15u;
	if (bulk != bytes) {     // final tile only; block-uniform
		if (threadIdx.x < (bytes - bulk) / 4)
			reinterpret_cast<uint32_t*>(tp + bulk)[threadIdx.x] =
				reinterpret_cast<const uint32_t*>(S + base * W + bulk)[threadIdx.x];
		__syncthreads();
	}
}

template <int ITEMS>
__device__ __forceinline__ void hjg_keys(const uint32_t* tw, uint32_t rows, uint32_t Ww, uint32_t kw, uint32_t kbytes,
		int warp, int lane, int64_t (&key)[ITEMS], bool (&valid)[ITEMS])
{
	#pragma unroll
	for (int j = 0; j < ITEMS; ++j) {
		const uint32_t p = warp * 32 * ITEMS + j * 32 + lane;
		valid[j] = p < rows;
		key[j] = 0;
		if (valid[j]) {
			const uint32_t* k = tw + p * Ww + kw;
			key[j] = kbytes == 4 ? (int64_t) (int32_t) k[0] : (int64_t) (((uint64_t) k[1] << 32) | k[0]);
		}
	}
}

template <bool MATERIALIZE, int MODE, int ITEMS>
__global__ void __launch_bounds__(HJG_THREADS, 2)
k_probe_staged(const char* __restrict__ S, uint64_t n, uint32_t W, uint32_t koff, uint32_t kbytes,
		const HjProbeTable tb, const HjWordMap wm, char* __restrict__ out, uint64_t out_cap,
		unsigned long long* __restrict__ cursor, unsigned long long* __restrict__ agg, int* __restrict__ status)
{
	constexpr uint32_t T = HJG_THREADS * ITEMS;
	extern __shared__ __align__(128) unsigned char sm[];
	// [HJG_BUFS tiles of T * W bytes][T build values][T tile rows (u16)]
	unsigned char* const tin0 = sm;
	uint64_t* const oval = reinterpret_cast<uint64_t*>(sm + (size_t) HJG_BUFS * T * W);
	uint16_t* const orow = reinterpret_cast<uint16_t*>(oval + T);
	__shared__ __align__(8) uint64_t bar[HJG_BUFS];
	__shared__ uint32_t wsum[HJG_WARPS];
	__shared__ uint8_t map[HJG_MAX_OW];
	__shared__ unsigned long long tile_at;
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const uint64_t ntiles = pg_div_up(n, T);
	const uint64_t keep = pg_policy_evict_last(), stream = pg_policy_evict_first();
	const uint32_t Ww = W >> 2, kw = koff >> 2, ow = wm.ow;
	// Copy-out shape: a row is upr store units of uw words; lane l of a warp
	// stores unit l % upr of row l / upr, so each warp step writes rpw whole
	// rows with one coalesced store and a lane's source words stay fixed.
	const uint32_t uw = wm.uw, upr = ow / uw, rpw = 32 / upr;
	const uint32_t my_row = lane / upr, my_unit = lane - my_row * upr;
	const bool copier = lane < rpw * upr;
	unsigned long long cnt_acc = 0, sum_acc = 0;
	#pragma unroll
	for (int i = 0; i < HJG_MAX_OW; ++i) if (tid == i) map[i] = wm.src[i];   // static indices: no local copy
	if (tid == 0) {
		#pragma unroll
		for (int b = 0; b < HJG_BUFS; ++b) pg_mbar_init(&bar[b], 1);
		pg_fence_mbar_init();
	}
	__syncthreads();
	const uint32_t src0 = copier ? map[my_unit * uw] : 0, src1 = copier && uw == 2 ? map[my_unit * uw + 1] : 0;
	const bool need_val = src0 >= 64 || (uw == 2 && src1 >= 64);
	uint64_t tile = blockIdx.x;
	if (tile >= ntiles) return;
	const uint64_t G = gridDim.x;
	// Software pipeline over the CTA's tiles t0, t1, t2, ... in buffers 0, 1,
	// 2, 0, ...: while tile t is ranked and written out, the table loads of
	// tile t + 1 are in flight and tile t + 2 is arriving. The copy of t + 2
	// is issued after tile t's first barrier, when every thread has finished
	// writing out tile t - 1, whose buffer it takes.
	if (tid == 0) {
		hjg_issue(S, n, W, T, tile, tin0, bar, 0, stream);
		if (tile + G < ntiles) hjg_issue(S, n, W, T, tile + G, tin0, bar, 1, stream);
	}
	uint32_t phases = 0;      // bit b: parity expected next on bar[b]
	int64_t key[ITEMS];
	bool valid[ITEMS];
	HjPending<MODE, ITEMS> pd;
	{
		const uint32_t rows = (uint32_t) pg_min64(T, n - tile * T);
		hjg_arrive(S, tile * T, rows, W, tin0, bar, 0, phases, status);
		hjg_keys<ITEMS>(reinterpret_cast<const uint32_t*>(tin0), rows, Ww, kw, kbytes, warp, lane, key, valid);
		hj_issue_items<MODE, ITEMS>(tb, key, valid, pd, keep);
	}
	for (int b = 0; tile < ntiles; tile += G, b = b == HJG_BUFS - 1 ? 0 : b + 1) {
		const int nb = b == HJG_BUFS - 1 ? 0 : b + 1, fb = nb == HJG_BUFS - 1 ? 0 : nb + 1;
		unsigned char* const tp = tin0 + (size_t) b * T * W;
		const uint32_t* const tw = reinterpret_cast<const uint32_t*>(tp);
		// Next tile: arrive, keys, table loads issued (used next iteration).
		int64_t nkey[ITEMS];
		bool nvalid[ITEMS];
		HjPending<MODE, ITEMS> npd;
		const bool has_next = tile + G < ntiles;
		if (has_next) {
			unsigned char* const np = tin0 + (size_t) nb * T * W;
			const uint32_t nrows = (uint32_t) pg_min64(T, n - (tile + G) * T);
			hjg_arrive(S, (tile + G) * T, nrows, W, np, bar, nb, phases, status);
			hjg_keys<ITEMS>(reinterpret_cast<const uint32_t*>(np), nrows, Ww, kw, kbytes, warp, lane, nkey, nvalid);
			hj_issue_items<MODE, ITEMS>(tb, nkey, nvalid, npd, keep);
		}
		bool hit[ITEMS];
		uint64_t val[ITEMS];
		hj_resolve_items<MODE, ITEMS>(tb, key, valid, pd, hit, val, keep);
		if (MATERIALIZE) {
			uint32_t ball[ITEMS], mine = 0;
			#pragma unroll
			for (int j = 0; j < ITEMS; ++j) { ball[j] = __ballot_sync(0xffffffffu, hit[j]); mine += __popc(ball[j]); }
			if (lane == 0) wsum[warp] = mine;
			__syncthreads();
			if (tid == 0 && tile + 2 * G < ntiles) hjg_issue(S, n, W, T, tile + 2 * G, tin0, bar, fb, stream);
			uint32_t pos = 0, total = 0;
			#pragma unroll
			for (int w = 0; w < HJG_WARPS; ++w) { const uint32_t c = wsum[w]; pos += w < warp ? c : 0; total += c; }
			if (tid == 0) tile_at = total ? atomicAdd(cursor, (unsigned long long) total) : 0;
			#pragma unroll
			for (int j = 0; j < ITEMS; ++j) {
				if (hit[j]) {
					const uint32_t q = pos + __popc(ball[j] & ((1u << lane) - 1));
					orow[q] = (uint16_t) (warp * 32 * ITEMS + j * 32 + lane);
					oval[q] = val[j];
				}
				pos += __popc(ball[j]);
			}
			__syncthreads();
			const unsigned long long at = tile_at;
			const uint64_t room = at < out_cap ? out_cap - at : 0;
			const uint32_t lim = (uint32_t) pg_min64(total, room);
			if (copier) {
				uint32_t* const dst = reinterpret_cast<uint32_t*>(out) + at * ow;
				for (uint32_t r = warp * rpw + my_row; r < lim; r += HJG_WARPS * rpw) {
					const uint32_t* const t = tw + orow[r] * Ww;
					const uint64_t bv = need_val ? oval[r] : 0;
					const uint32_t a = hjg_word(t, bv, src0);
					if (uw == 2)
						__stcs(reinterpret_cast<uint2*>(dst + r * ow) + my_unit, make_uint2(a, hjg_word(t, bv, src1)));
					else
						__stcs(dst + r * ow + my_unit, a);
				}
			}
		} else {
			#pragma unroll
			for (int j = 0; j < ITEMS; ++j) {
				if (!hit[j]) continue;
				cnt_acc++;
				if (wm.sum_words) {
					const uint32_t* t = tw + (warp * 32 * ITEMS + j * 32 + lane) * Ww;
					const uint32_t lo = hjg_word(t, val[j], map[wm.sum_w0]);
					if (wm.sum_words == 2)
						sum_acc += ((unsigned long long) hjg_word(t, val[j], map[wm.sum_w0 + 1]) << 32) | lo;
					else sum_acc += (unsigned long long) (long long) (int32_t) lo;
				}
			}
			__syncthreads();   // every thread is done with this tile's buffer
			if (tid == 0 && tile + 2 * G < ntiles) hjg_issue(S, n, W, T, tile + 2 * G, tin0, bar, fb, stream);
		}
		if (has_next) {
			#pragma unroll
			for (int j = 0; j < ITEMS; ++j) { key[j] = nkey[j]; valid[j] = nvalid[j]; }
			pd = npd;
		}
	}
	if (!MATERIALIZE) {
		#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			cnt_acc += __shfl_down_sync(0xffffffffu, cnt_acc, o);
			sum_acc += __shfl_down_sync(0xffffffffu, sum_acc, o);
		}
		if (lane == 0) { atomicAdd(&agg[0], cnt_acc); atomicAdd(&agg[1], sum_acc); }
	}
}

// ---------------------------------------------------------------------------
// Unique-key probe of 16-byte tuples without block barriers: every warp runs
// on its own. Warp w of the grid owns blocks w, w + W, w + 2W, ... of
// 32 * ITEMS probe tuples; each block arrives in the warp's own shared-memory
// stage by a bulk copy (2 stages in flight per warp, L2 evict-first), and
// every lane has ITEMS table lookups in flight at once. With unique build keys
// a probe tuple yields at most one row, so the 128-tuple chunk c writes its
// rows to output rows [128c, 128c + matches) in probe order: no atomics and no
// block-wide ranking. When every probe tuple matches (PK-FK) the output is
// already dense; otherwise per-chunk counts drive a compaction pass.
// Dense tables larger than L2 holds next to the streams are probed in two
// passes over the probe relation, each looking up only keys whose table index
// d lies in [dlo, dhi) (half the table, which stays in L2): run 0 writes a
// chunk's rows at its front and counts them in the low word of the chunk's
// count, run 1 writes them backwards from the chunk's end and counts them in
// the high word; run -1 is the single pass over the whole table.
// ---------------------------------------------------------------------------
#define PW_WARPS 8
#define PW_CHUNK 128
#define PW_STAGES 2

template <bool MATERIALIZE, int MODE, int ITEMS>
__global__ void __launch_bounds__(PW_WARPS * 32, MODE != 0 ? (ITEMS > 4 ? 3 : 4) : 2)
k_probe16_warp(const char* __restrict__ S, uint64_t n, uint32_t koff, const HjProbeTable tb,
		uint32_t wsel, uint32_t sum_w0, uint32_t sum_words, char* __restrict__ out,
		uint64_t* __restrict__ chunk_counts, unsigned long long* __restrict__ agg,
		int sum_col, int* __restrict__ status, uint64_t dlo, uint64_t dhi, int run)
{
	static_assert(ITEMS % 4 == 0, "a block is whole 128-tuple chunks");
	constexpr int BLK = 32 * ITEMS;                  // tuples per warp block
	constexpr int SUB = ITEMS / 4;                   // 128-tuple chunks per block
	constexpr int GROUP = MODE != 0 ? ITEMS : 4;     // lookups issued together (registers)
	extern __shared__ __align__(128) unsigned char sm[];
	__shared__ __align__(8) uint64_t bars[PW_WARPS][PW_STAGES];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	uint4* const st0 = reinterpret_cast<uint4*>(sm) + (size_t) warp * PW_STAGES * BLK;
	uint64_t* const bar = bars[warp];
	const uint64_t nchunks = pg_div_up(n, BLK);
	const uint64_t nchunks128 = pg_div_up(n, PW_CHUNK);
	const uint64_t W = (uint64_t) gridDim.x * PW_WARPS;
	const uint64_t first = (uint64_t) blockIdx.x * PW_WARPS + warp;
	const uint64_t mask = (1ull << tb.log2cap) - 1;
	const uint32_t tp_ = tb.cache & 3;
	const uint64_t keep = tp_ == 0 ? pg_policy_keep((tb.cache >> 4) & 7) : tp_ == 1 ? pg_policy_evict_normal()
		: tp_ == 2 ? pg_policy_evict_unchanged() : pg_policy_evict_first();
	const uint64_t instream = (tb.cache & 4) ? pg_policy_evict_normal() : pg_policy_evict_first();
	const uint64_t stream = (tb.cache & 8) ? pg_policy_evict_normal() : pg_policy_evict_first();
	const uint32_t w0 = wsel & 15, w1 = (wsel >> 4) & 15, w2 = (wsel >> 8) & 15, w3 = (wsel >> 12) & 15;
	unsigned long long cnt_acc = 0, sum_acc = 0;
	if (first >= nchunks) return;
	auto issue = [&](uint64_t c, int stg) {
		const uint32_t rows = (uint32_t) pg_min64(BLK, n - c * BLK);
		pg_mbar_expect_tx(&bar[stg], rows * 16);
		pg_bulk_g2s_hint(st0 + stg * BLK, S + c * (uint64_t) BLK * 16, rows * 16, &bar[stg], instream);
	};
	if (lane == 0) {
		for (int i = 0; i < PW_STAGES; ++i) pg_mbar_init(&bar[i], 1);
		pg_fence_mbar_init();
		for (int i = 0; i < PW_STAGES; ++i)
			if (first + i * W < nchunks) issue(first + i * W, i);
	}
	__syncwarp();
	const uint32_t spin = pg_spin_knob(status);
	for (uint64_t k = 0, c = first; c < nchunks; ++k, c += W) {
		const int stg = (int) (k % PW_STAGES);
		const uint32_t parity = (uint32_t) ((k / PW_STAGES) & 1);
		// A wait past the context's limit records PG_ERR_TIMEOUT and drains
		// the copy; if even that gives up the chunk is unspecified, all
		// accesses stay in bounds and the host reads the status.
		pg_mbar_wait_timed(&bar[stg], parity, spin, status);
		const uint4* const tp = st0 + stg * BLK;
		const uint32_t rows = (uint32_t) pg_min64(BLK, n - c * BLK);
		uint32_t rank[SUB];
		#pragma unroll
		for (int q = 0; q < SUB; ++q) rank[q] = 0;
		#pragma unroll
		for (int g = 0; g < ITEMS; g += GROUP) {
			int64_t key[GROUP];
			uint64_t val[GROUP];
			bool hit[GROUP];
			if (MODE != 0) {
				uint32_t bits[GROUP];
				#pragma unroll
				for (int j = 0; j < GROUP; ++j) {
					const uint32_t p = (g + j) * 32 + lane;
					hit[j] = false; val[j] = 0; bits[j] = 0;
					if (p < rows) {
						const uint4 t = tp[p];
						key[j] = koff == 0 ? (int64_t) (((uint64_t) t.y << 32) | t.x) : (int64_t) (((uint64_t) t.w << 32) | t.z);
						const unsigned long long d = (unsigned long long) key[j] - (unsigned long long) tb.dmin;
						if (d >= dlo && d < dhi) {
							if (MODE == 2) {
								uint32_t e;
								asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;"
										: "=r"(e) : "l"(tb.dense32 + d), "l"(keep));
								bits[j] = e != 0xFFFFFFFFu;
								val[j] = tb.vmin + e;
							} else {
								bits[j] = __ldg(tb.dense_bits + (d >> 5)) >> (d & 31);
								asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u64 %0, [%1], %2;"
										: "=l"(val[j]) : "l"(tb.dense_val + d), "l"(keep));
							}
							hit[j] = true;
						}
					}
				}
				#pragma unroll
				for (int j = 0; j < GROUP; ++j) hit[j] = hit[j] && (bits[j] & 1);
			} else {
				uint64_t slot[GROUP];
				bool open[GROUP];
				#pragma unroll
				for (int j = 0; j < GROUP; ++j) {
					const uint32_t p = (g + j) * 32 + lane;
					hit[j] = false; open[j] = false; val[j] = 0; key[j] = 0;
					if (p < rows) {
						const uint4 t = tp[p];
						key[j] = koff == 0 ? (int64_t) (((uint64_t) t.y << 32) | t.x) : (int64_t) (((uint64_t) t.w << 32) | t.z);
						if (key[j] == PG_EMPTY_KEY) { if (tb.nside) { hit[j] = true; val[j] = tb.side[0]; } }
						else { open[j] = true; slot[j] = hj_slot0(key[j], tb.log2cap); }
					}
				}
				for (uint32_t round = 0; round <= (mask >> 1); ++round) {
					pg_u64x4 bk[GROUP];
					bool any = false;
					#pragma unroll
					for (int j = 0; j < GROUP; ++j)
						if (open[j]) { bk[j] = pg_ld_bucket32(tb.slots + 2 * slot[j], keep); any = true; }
					if (!any) break;
					#pragma unroll
					for (int j = 0; j < GROUP; ++j) {
						if (!open[j]) continue;
						if ((long long) bk[j].a == key[j]) { hit[j] = true; val[j] = bk[j].b; open[j] = false; }
						else if (bk[j].a == (unsigned long long) PG_EMPTY_KEY) open[j] = false;
						else if ((long long) bk[j].c == key[j]) { hit[j] = true; val[j] = bk[j].d; open[j] = false; }
						else if (bk[j].c == (unsigned long long) PG_EMPTY_KEY) open[j] = false;
						else slot[j] = (slot[j] + 2) & mask;
					}
				}
			}
			#pragma unroll
			for (int j = 0; j < GROUP; ++j) {
				const int q = (g + j) / 4;               // 128-tuple chunk within the block
				const uint32_t ball = __ballot_sync(0xffffffffu, hit[j]);
				if (hit[j]) {
					const uint4 t = tp[(g + j) * 32 + lane];
					if (MATERIALIZE) {
						const uint32_t r = rank[q] + __popc(ball & ((1u << lane) - 1));
						const uint64_t c0 = c * BLK + q * PW_CHUNK;
						const uint64_t row = run == 1 ? c0 + pg_min64(PW_CHUNK, n - c0) - 1 - r : c0 + r;
						pg_st_hint16(out + row * 16, make_uint4(hj_pick(t, val[j], w0), hj_pick(t, val[j], w1),
								hj_pick(t, val[j], w2), hj_pick(t, val[j], w3)), stream);
					} else if (sum_col >= 0) {
						const uint32_t lo = hj_pick(t, val[j], (wsel >> (4 * sum_w0)) & 15);
						if (sum_words == 2)
							sum_acc += ((unsigned long long) hj_pick(t, val[j], (wsel >> (4 * sum_w0 + 4)) & 15) << 32) | lo;
						else sum_acc += (unsigned long long) (long long) (int32_t) lo;
					}
				}
				rank[q] += __popc(ball);
			}
		}
		#pragma unroll
		for (int q = 0; q < SUB; ++q) {
			cnt_acc += rank[q];
			if (MATERIALIZE && lane == 0 && c * SUB + q < nchunks128) {
				if (run < 0) chunk_counts[c * SUB + q] = rank[q];
				else reinterpret_cast<uint32_t*>(chunk_counts)[2 * (c * SUB + q) + run] = rank[q];
			}
		}
		// Every lane has finished reading this stage: refill it.
		__syncwarp();
		if (lane == 0 && c + PW_STAGES * W < nchunks) issue(c + PW_STAGES * W, stg);
	}
	if (!MATERIALIZE) {
		#pragma unroll
		for (int o = 16; o > 0; o >>= 1) sum_acc += __shfl_down_sync(0xffffffffu, sum_acc, o);
	}
	if (lane == 0) { atomicAdd(&agg[0], cnt_acc); if (!MATERIALIZE) atomicAdd(&agg[1], sum_acc); }
}

// ---------------------------------------------------------------------------
// Dense-table probe of 16-byte tuples straight from global memory into
// registers: the same warp-owned 128-tuple chunks, positional output and
// two-pass runs as k_probe16_warp, but each lane loads its four tuples with
// 16-byte loads (a warp instruction covers 512 contiguous bytes) and the next
// chunk's loads are issued before the current chunk's table lookups, so a
// warp keeps eight tuple loads and four lookups in flight without shared
// memory or barriers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint4 hj_ld_stream(const char* p, uint64_t pol)
{
	uint4 v;
	asm("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
			: "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p), "l"(pol));
	return v;
}

__device__ __forceinline__ void hj_st_stream(char* p, uint4 v, uint64_t pol)
{
	asm volatile("st.global.L1::no_allocate.L2::cache_hint.v4.u32 [%0], {%1,%2,%3,%4}, %5;"
			:: "l"(p), "r"(v.x), "r"(v.y), "r"(v.z), "r"(v.w), "l"(pol));
}

// STD: the output row is (probe words 2-3, value) = the (P$1, B$1) projection
// of 16-byte tuples, picked without the general word selector.
// PRED: probe tuples failing the predicates `pr` skip their lookup (a Filter
// on the probe side run as the probe's prologue).
template <bool MATERIALIZE, int MODE, bool PF, bool STD = false, bool PRED = false>
__global__ void __launch_bounds__(PW_WARPS * 32, PF ? 4 : 5)
k_probe16_direct(const char* __restrict__ S, uint64_t n, uint32_t koff, const HjProbeTable tb0,
		uint32_t wsel, uint32_t sum_w0, uint32_t sum_words, char* __restrict__ out,
		uint64_t* __restrict__ chunk_counts, unsigned long long* __restrict__ agg,
		int sum_col, uint64_t dlo, uint64_t dhi, int run, const PgPred16 pr = PgPred16())
{
	static_assert(MODE == 1 || MODE == 2, "dense tables only");
	HjProbeTable tb = tb0;
	if (!hj_spec_resolve(tb)) return;
	// A speculative table is probed in one pass over its window: the host
	// passed the allocation's capacity, past the entries the build filled.
	if (tb0.hdr) { dlo = 0; dhi = tb.drange; }
	constexpr int ITEMS = PW_CHUNK / 32;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint64_t nchunks = pg_div_up(n, PW_CHUNK);
	const uint64_t W = (uint64_t) gridDim.x * PW_WARPS;
	const uint64_t first = (uint64_t) blockIdx.x * PW_WARPS + warp;
	const uint32_t tp_ = tb.cache & 3;
	const uint64_t keep = tp_ == 0 ? pg_policy_keep((tb.cache >> 4) & 7) : tp_ == 1 ? pg_policy_evict_normal()
		: tp_ == 2 ? pg_policy_evict_unchanged() : pg_policy_evict_first();
	const uint64_t instream = (tb.cache & 4) ? pg_policy_evict_normal() : pg_policy_evict_first();
	const uint64_t stream = (tb.cache & 8) ? pg_policy_evict_normal() : pg_policy_evict_first();
	const uint32_t w0 = wsel & 15, w1 = (wsel >> 4) & 15, w2 = (wsel >> 8) & 15, w3 = (wsel >> 12) & 15;
	unsigned long long cnt_acc = 0, sum_acc = 0;
	// Warps past the last chunk load nothing but still join the block's sum.
	const bool busy = first < nchunks;
	uint4 cur[ITEMS], nxt[ITEMS];
	auto load = [&](uint64_t c, uint4 (&t)[ITEMS]) {
		const uint32_t rows = (uint32_t) pg_min64(PW_CHUNK, n - c * PW_CHUNK);
		#pragma unroll
		for (int j = 0; j < ITEMS; ++j) {
			const uint32_t p = j * 32 + lane;
			t[j] = p < rows ? hj_ld_stream(S + (c * PW_CHUNK + p) * 16, instream) : make_uint4(0, 0, 0, 0);
		}
	};
	if (PF && busy) load(first, cur);
	for (uint64_t c = first; c < nchunks; c += W) {
		if (PF) { if (c + W < nchunks) load(c + W, nxt); }
		else load(c, cur);
		const uint32_t rows = (uint32_t) pg_min64(PW_CHUNK, n - c * PW_CHUNK);
		// Narrow tables keep the 4-byte entry (all ones: absent); wide ones
		// the 8-byte value and the presence bit.
		uint32_t e32[ITEMS], pres[ITEMS];
		uint64_t v64[ITEMS];
		#pragma unroll
		for (int j = 0; j < ITEMS; ++j) {
			const uint32_t p = j * 32 + lane;
			e32[j] = 0xFFFFFFFFu; pres[j] = 0; v64[j] = 0;
			const uint4 t = cur[j];
			const int64_t key = koff == 0 ? (int64_t) (((uint64_t) t.y << 32) | t.x) : (int64_t) (((uint64_t) t.w << 32) | t.z);
			const unsigned long long d = (unsigned long long) key - (unsigned long long) tb.dmin;
			if (p < rows && d >= dlo && d < dhi && (!PRED || pg_pred16(pr, t))) {
				if (MODE == 2) {
					if (tb.cache & 128)
						asm("ld.global.nc.L1::evict_last.L2::cache_hint.u32 %0, [%1], %2;"
								: "=r"(e32[j]) : "l"(tb.dense32 + d), "l"(keep));
					else
						asm("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;"
								: "=r"(e32[j]) : "l"(tb.dense32 + d), "l"(keep));
				} else {
					pres[j] = __ldg(tb.dense_bits + (d >> 5)) >> (d & 31);
					asm("ld.global.nc.L1::no_allocate.L2::cache_hint.u64 %0, [%1], %2;"
							: "=l"(v64[j]) : "l"(tb.dense_val + d), "l"(keep));
				}
			}
		}
		uint32_t rank = 0;
		#pragma unroll
		for (int j = 0; j < ITEMS; ++j) {
			const bool h = MODE == 2 ? e32[j] != 0xFFFFFFFFu : (pres[j] & 1) != 0;
			const uint32_t ball = __ballot_sync(0xffffffffu, h);
			if (h) {
				const uint64_t v = MODE == 2 ? tb.vmin + e32[j] : v64[j];
				const uint4 t = cur[j];
				if (MATERIALIZE) {
					const uint32_t r = rank + __popc(ball & ((1u << lane) - 1));
					const uint64_t row = run == 1 ? c * PW_CHUNK + rows - 1 - r : c * PW_CHUNK + r;
					if (STD)
						hj_st_stream(out + row * 16, make_uint4(t.z, t.w, (uint32_t) v, (uint32_t) (v >> 32)), stream);
					else
						hj_st_stream(out + row * 16, make_uint4(hj_pick(t, v, w0), hj_pick(t, v, w1),
								hj_pick(t, v, w2), hj_pick(t, v, w3)), stream);
				} else if (sum_col >= 0) {
					const uint32_t lo = hj_pick(t, v, (wsel >> (4 * sum_w0)) & 15);
					if (sum_words == 2)
						sum_acc += ((unsigned long long) hj_pick(t, v, (wsel >> (4 * sum_w0 + 4)) & 15) << 32) | lo;
					else sum_acc += (unsigned long long) (long long) (int32_t) lo;
				}
			}
			rank += __popc(ball);
		}
		cnt_acc += rank;
		if (MATERIALIZE && lane == 0) {
			if (run < 0) chunk_counts[c] = rank;
			else reinterpret_cast<uint32_t*>(chunk_counts)[2 * c + run] = rank;
		}
		if (PF) {
			#pragma unroll
			for (int j = 0; j < ITEMS; ++j) cur[j] = nxt[j];
		}
	}
	if (!MATERIALIZE) {
		#pragma unroll
		for (int o = 16; o > 0; o >>= 1) sum_acc += __shfl_down_sync(0xffffffffu, sum_acc, o);
	}
	// One pair of global atomics per CTA: thousands of warps adding into the
	// same two words queue up at one L2 slice, which on short probes (16M
	// tuples) was a good part of the kernel's time.
	__shared__ unsigned long long red[2][PW_WARPS];
	if (lane == 0) { red[0][warp] = cnt_acc; red[1][warp] = sum_acc; }
	__syncthreads();
	if (threadIdx.x == 0) {
		unsigned long long c = 0, t = 0;
		#pragma unroll
		for (int w = 0; w < PW_WARPS; ++w) { c += red[0][w]; t += red[1][w]; }
		if (c) atomicAdd(&agg[0], c);
		if (!MATERIALIZE && t) atomicAdd(&agg[1], t);
	}
}

// ---------------------------------------------------------------------------
// Deeper pipeline of the narrow dense probe (standard 16-byte output rows):
// while chunk c's rows are written, the table lookups of chunk c + W are in
// flight and the tuples of chunk c + 2W are loading, so lookup latency and
// stream latency both overlap with the stores of another chunk.
// ---------------------------------------------------------------------------
template <bool PRED>
__device__ __forceinline__ void hj_lookup4(const HjProbeTable& tb, const uint4 (&t)[4], uint32_t rows, int lane,
		uint32_t koff, uint64_t keep, uint32_t (&e)[4], const PgPred16& pr)
{
	#pragma unroll
	for (int j = 0; j < 4; ++j) {
		const int64_t key = koff == 0 ? (int64_t) (((uint64_t) t[j].y << 32) | t[j].x)
			: (int64_t) (((uint64_t) t[j].w << 32) | t[j].z);
		const unsigned long long d = (unsigned long long) key - (unsigned long long) tb.dmin;
		e[j] = 0xFFFFFFFFu;
		if ((uint32_t) (j * 32 + lane) < rows && d < tb.drange && (!PRED || pg_pred16(pr, t[j]))) {
			if (tb.cache & 128)
				asm("ld.global.nc.L1::evict_last.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(e[j]) : "l"(tb.dense32 + d), "l"(keep));
			else
				asm("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(e[j]) : "l"(tb.dense32 + d), "l"(keep));
		}
	}
}

template <bool PRED>
__global__ void __launch_bounds__(PW_WARPS * 32, 4)
k_probe16_deep(const char* __restrict__ S, uint64_t n, uint32_t koff, const HjProbeTable tb0, char* __restrict__ out,
		uint64_t* __restrict__ chunk_counts, unsigned long long* __restrict__ agg, const PgPred16 pr)
{
	HjProbeTable tb = tb0;
	if (!hj_spec_resolve(tb)) return;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint64_t nchunks = pg_div_up(n, PW_CHUNK);
	const uint64_t W = (uint64_t) gridDim.x * PW_WARPS;
	const uint64_t first = (uint64_t) blockIdx.x * PW_WARPS + warp;
	const uint64_t keep = pg_policy_keep((tb.cache >> 4) & 7);
	const uint64_t stream = pg_policy_evict_first();
	unsigned long long cnt_acc = 0;
	if (first >= nchunks) return;
	auto rows_of = [&](uint64_t c) -> uint32_t { return (uint32_t) pg_min64(PW_CHUNK, n - c * PW_CHUNK); };
	auto load = [&](uint64_t c, uint4 (&t)[4]) {
		const uint32_t rows = c < nchunks ? rows_of(c) : 0;
		#pragma unroll
		for (int j = 0; j < 4; ++j) {
			const uint32_t p = j * 32 + lane;
			t[j] = p < rows ? hj_ld_stream(S + (c * PW_CHUNK + p) * 16, stream) : make_uint4(0, 0, 0, 0);
		}
	};
	uint4 cur[4], nxt[4], nx2[4];
	uint32_t ecur[4], enxt[4];
	load(first, cur);
	load(first + W, nxt);
	hj_lookup4<PRED>(tb, cur, rows_of(first), lane, koff, keep, ecur, pr);
	for (uint64_t c = first; c < nchunks; c += W) {
		const uint64_t c1 = c + W, c2 = c + 2 * W;
		if (c1 < nchunks) hj_lookup4<PRED>(tb, nxt, rows_of(c1), lane, koff, keep, enxt, pr);
		load(c2, nx2);
		const uint32_t rows = rows_of(c);
		uint32_t rank = 0;
		#pragma unroll
		for (int j = 0; j < 4; ++j) {
			const bool h = ecur[j] != 0xFFFFFFFFu;
			const uint32_t ball = __ballot_sync(0xffffffffu, h);
			if (h) {
				const uint64_t v = tb.vmin + ecur[j];
				const uint64_t row = c * PW_CHUNK + rank + __popc(ball & ((1u << lane) - 1));
				hj_st_stream(out + row * 16, make_uint4(cur[j].z, cur[j].w, (uint32_t) v, (uint32_t) (v >> 32)), stream);
			}
			rank += __popc(ball);
		}
		(void) rows;
		cnt_acc += rank;
		if (lane == 0) chunk_counts[c] = rank;
		#pragma unroll
		for (int j = 0; j < 4; ++j) { cur[j] = nxt[j]; nxt[j] = nx2[j]; ecur[j] = enxt[j]; }
	}
	if (lane == 0) atomicAdd(&agg[0], cnt_acc);
}

// Compacting form of the deep pipeline, for probes where a fraction of the
// probe tuples yields rows (a Filter fused into the probe): each warp appends
// its rows to a 512-row stage in shared memory and, before a chunk could
// overflow it, reserves an output range with one atomicAdd on `cursor` and
// writes the stage out with coalesced 16-byte stores. One pass, no positional
// rows to compact afterwards; row order is unspecified (as for every join
// output). Rows past `cap` are counted but not written.
#define HJ_STAGE_ROWS 512
// STD: (P$1, B$1) rows, picked without the word selector.
template <bool PRED, bool STD>
__global__ void __launch_bounds__(PW_WARPS * 32, 3)
k_probe16_stage(const char* __restrict__ S, uint64_t n, uint32_t koff, const HjProbeTable tb, uint32_t wsel,
		char* __restrict__ out, uint64_t cap, unsigned long long* __restrict__ cursor, const PgPred16 pr)
{
	extern __shared__ uint4 hj_stage[];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	uint4* stage = hj_stage + warp * HJ_STAGE_ROWS;
	const uint64_t nchunks = pg_div_up(n, PW_CHUNK);
	const uint64_t W = (uint64_t) gridDim.x * PW_WARPS;
	const uint64_t first = (uint64_t) blockIdx.x * PW_WARPS + warp;
	const uint64_t keep = pg_policy_evict_last();
	const uint64_t stream = pg_policy_evict_first();
	const uint32_t w0 = wsel & 15, w1 = (wsel >> 4) & 15, w2 = (wsel >> 8) & 15, w3 = (wsel >> 12) & 15;
	if (first >= nchunks) return;
	auto rows_of = [&](uint64_t c) -> uint32_t { return (uint32_t) pg_min64(PW_CHUNK, n - c * PW_CHUNK); };
	auto load = [&](uint64_t c, uint4 (&t)[4]) {
		const uint32_t rows = c < nchunks ? rows_of(c) : 0;
		#pragma unroll
		for (int j = 0; j < 4; ++j) {
			const uint32_t p = j * 32 + lane;
			t[j] = p < rows ? hj_ld_stream(S + (c * PW_CHUNK + p) * 16, stream) : make_uint4(0, 0, 0, 0);
		}
	};
	uint32_t fill = 0;
	auto flush = [&]() {
		unsigned long long base = 0;
		if (lane == 0) base = atomicAdd(cursor, (unsigned long long) fill);
		base = __shfl_sync(0xffffffffu, base, 0);
		__syncwarp();
		for (uint32_t i = lane; i < fill; i += 32)
			if (base + i < cap) hj_st_stream(out + (base + i) * 16, stage[i], stream);
		__syncwarp();
		fill = 0;
	};
	uint4 cur[4], nxt[4], nx2[4];
	uint32_t ecur[4], enxt[4];
	load(first, cur);
	load(first + W, nxt);
	hj_lookup4<PRED>(tb, cur, rows_of(first), lane, koff, keep, ecur, pr);
	for (uint64_t c = first; c < nchunks; c += W) {
		const uint64_t c1 = c + W, c2 = c + 2 * W;
		if (c1 < nchunks) hj_lookup4<PRED>(tb, nxt, rows_of(c1), lane, koff, keep, enxt, pr);
		load(c2, nx2);
		uint32_t rank = 0;
		#pragma unroll
		for (int j = 0; j < 4; ++j) {
			const bool h = ecur[j] != 0xFFFFFFFFu;
			const uint32_t ball = __ballot_sync(0xffffffffu, h);
			if (h) {
				const uint64_t v = tb.vmin + ecur[j];
				const uint4 t = cur[j];
				stage[fill + rank + __popc(ball & ((1u << lane) - 1))] = STD
					? make_uint4(t.z, t.w, (uint32_t) v, (uint32_t) (v >> 32))
					: make_uint4(hj_pick(t, v, w0), hj_pick(t, v, w1), hj_pick(t, v, w2), hj_pick(t, v, w3));
			}
			rank += __popc(ball);
		}
		fill += rank;
		if (fill > HJ_STAGE_ROWS - PW_CHUNK) flush();
		#pragma unroll
		for (int j = 0; j < 4; ++j) { cur[j] = nxt[j]; nxt[j] = nx2[j]; ecur[j] = enxt[j]; }
	}
	if (fill) flush();
}

// Positional probe output: the 128-tuple chunk c (rows_c = min(128, n - 128c)
// probe tuples) holds lo = counts[c] & 0xffffffff rows at its front,
// [128c, 128c + lo), and hi = counts[c] >> 32 rows at its back,
// [128c + rows_c - hi, 128c + rows_c). k_chunk_totals turns the counts into
// lo + hi; k_compact_chunks moves both runs of chunk c to
// [offs[c], offs[c] + lo + hi) of `dst`.
// Front and back run lengths of chunk c, clamped to the chunk's rows.
__device__ __forceinline__ void hj_chunk_runs(uint64_t cnt, uint64_t n, uint64_t c, uint32_t& lo, uint32_t& hi,
		uint32_t& rows)
{
	rows = (uint32_t) pg_min64(PW_CHUNK, n - c * PW_CHUNK);
	lo = pg_min32((uint32_t) cnt, rows);
	hi = pg_min32((uint32_t) (cnt >> 32), rows - lo);
}

__global__ void k_chunk_totals(const uint64_t* __restrict__ counts, uint64_t* __restrict__ tot, uint64_t nchunks,
		uint64_t n)
{
	for (uint64_t c = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; c < nchunks; c += (uint64_t) gridDim.x * blockDim.x) {
		uint32_t lo, hi, rows;
		hj_chunk_runs(counts[c], n, c, lo, hi, rows);
		tot[c] = lo + hi;
	}
}

__global__ void k_compact_chunks(const uint4* __restrict__ src, const uint64_t* __restrict__ counts,
		const uint64_t* __restrict__ offs, uint64_t nchunks, uint64_t n, uint4* __restrict__ dst, uint64_t cap)
{
	for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
		uint32_t lo, hi, rows;
		hj_chunk_runs(counts[c], n, c, lo, hi, rows);
		const uint64_t o = offs[c];
		for (uint32_t i = threadIdx.x; i < lo + hi; i += blockDim.x)
			if (o + i < cap) dst[o + i] = src[c * PW_CHUNK + (i < lo ? i : rows - hi + (i - lo))];
	}
}

// ---------------------------------------------------------------------------
// General probe (duplicate build keys and/or row-index values): pass 1 counts
// matches per tile (and folds count/sum), pass 2 writes at scanned offsets.
// ---------------------------------------------------------------------------
template <bool WRITE>
__global__ void __launch_bounds__(HJ_THREADS)
k_probe_general(const char* __restrict__ S, uint64_t n, uint32_t W, uint32_t koff, uint32_t kbytes,
		const unsigned long long* __restrict__ slots, uint32_t log2cap,
		const unsigned long long* __restrict__ side, uint32_t nside,
		HjCols pc, bool inline_val, const char* __restrict__ R, uint32_t wR,
		uint64_t* __restrict__ tile_counts, char* __restrict__ out,
		unsigned long long* __restrict__ agg, int sum_col, int* __restrict__ status)
{
	__shared__ unsigned long long wtot[HJ_THREADS / 32];
	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const uint64_t mask = (1ull << log2cap) - 1;
	const uint64_t ntiles = pg_div_up(n, HJ_TILE);
	unsigned long long cnt_acc = 0, sum_acc = 0;
	const uint64_t ow = (uint64_t) pc.ow_words * 4;

	for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
		const uint64_t base = tile * HJ_TILE;
		unsigned long long run = WRITE ? tile_counts[tile] : 0;
		#pragma unroll 1
		for (int j = 0; j < HJ_ITEMS; ++j) {
			uint64_t r = base + (uint64_t) j * HJ_THREADS + tid;
			const char* pt = S + r * W;
			uint32_t c = 0;
			int64_t k = 0;
			if (r < n) {
				k = pg_load_key(pt + koff, kbytes);
				if (k == PG_EMPTY_KEY) c = nside;
				else {
					uint64_t s = hj_slot0(k, log2cap);
					for (uint64_t probe = 0; probe <= mask; ++probe) {
						uint4 v = pg_ld_table16(slots + 2 * s);
						int64_t sk = (int64_t) (((uint64_t) v.y << 32) | v.x);
						if (sk == PG_EMPTY_KEY) break;
						if (sk == k) {
							if (!WRITE && sum_col >= 0) {
								uint64_t val = ((uint64_t) v.w << 32) | v.z;
								uint32_t lo = hj_out_word(pc, sum_col, 0, pt, val, inline_val, R, wR);
								if (pc.words[sum_col] == 2) {
									uint32_t hi = hj_out_word(pc, sum_col, 1, pt, val, inline_val, R, wR);
									sum_acc += ((unsigned long long) hi << 32) | lo;
								} else sum_acc += (unsigned long long) (long long) (int32_t) lo;
							}
							++c;
						}
						s = (s + 1) & mask;
					}
				}
			}
			if (!WRITE && sum_col >= 0 && k == PG_EMPTY_KEY && r < n) {
				for (uint32_t q = 0; q < nside; ++q) {
					uint64_t val = side[q];
					uint32_t lo = hj_out_word(pc, sum_col, 0, pt, val, inline_val, R, wR);
					if (pc.words[sum_col] == 2) {
						uint32_t hi = hj_out_word(pc, sum_col, 1, pt, val, inline_val, R, wR);
						sum_acc += ((unsigned long long) hi << 32) | lo;
					} else sum_acc += (unsigned long long) (long long) (int32_t) lo;
				}
			}
			cnt_acc += c;
			if (WRITE) {
				// Exclusive block scan of c in (item, warp, lane) order.
				unsigned long long x = c;
				#pragma unroll
				for (int o = 1; o < 32; o <<= 1) {
					unsigned long long y = __shfl_up_sync(0xffffffffu, x, o);
					if (lane >= o) x += y;
				}
				if (lane == 31) wtot[warp] = x;
				__syncthreads();
				unsigned long long before = 0, total = 0;
				for (int w = 0; w < HJ_THREADS / 32; ++w) { if (w < warp) before += wtot[w]; total += wtot[w]; }
				unsigned long long pos = run + before + x - c;
				run += total;
				__syncthreads();
				if (c && r < n) {
					auto emit = [&](uint64_t val) {
						uint32_t* o = reinterpret_cast<uint32_t*>(out + pos * ow);
						int wo = 0;
						for (int cc = 0; cc < pc.n; ++cc)
							for (int q = 0; q < pc.words[cc]; ++q)
								o[wo++] = hj_out_word(pc, cc, q, pt, val, inline_val, R, wR);
						++pos;
					};
					if (k == PG_EMPTY_KEY) {
						for (uint32_t q = 0; q < nside; ++q) emit(side[q]);
					} else {
						uint64_t s = hj_slot0(k, log2cap);
						for (uint64_t probe = 0; probe <= mask; ++probe) {
							uint4 v = pg_ld_table16(slots + 2 * s);
							int64_t sk = (int64_t) (((uint64_t) v.y << 32) | v.x);
							if (sk == PG_EMPTY_KEY) break;
							if (sk == k) emit(((uint64_t) v.w << 32) | v.z);
							s = (s + 1) & mask;
						}
					}
				}
			}
		}
	}
	if (!WRITE) {
		// The host launches one CTA per tile, so the CTA total is the tile's.
		#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			cnt_acc += __shfl_down_sync(0xffffffffu, cnt_acc, o);
			sum_acc += __shfl_down_sync(0xffffffffu, sum_acc, o);
		}
		if (lane == 0) wtot[warp] = cnt_acc;
		__syncthreads();
		if (tid == 0) {
			unsigned long long t = 0;
			for (int w = 0; w < HJ_THREADS / 32; ++w) t += wtot[w];
			tile_counts[blockIdx.x] = t;
		}
		if (lane == 0) { atomicAdd(&agg[0], cnt_acc); atomicAdd(&agg[1], sum_acc); }
	}
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static int hj_validate_rel(pg_ctx* ctx, const pg_rel* r, const char* who)
{
	if (!r) return pg_fail(ctx, PG_ERR_ARG, std::string(who) + ": null relation");
	if (r->n && !r->data) return pg_fail(ctx, PG_ERR_ARG, std::string(who) + ": null data");
	if (r->width == 0 || (r->width & 3))
		return pg_fail(ctx, PG_ERR_UNSUPPORTED, std::string(who) + ": tuple width must be a multiple of 4 bytes");
	if ((r->key_bytes != 4 && r->key_bytes != 8) || (r->key_off & 3) || r->key_off + r->key_bytes > r->width)
		return pg_fail(ctx, PG_ERR_ARG, std::string(who) + ": key must be a 4-byte-aligned int or long column");
	if (r->n && (reinterpret_cast<uintptr_t>(r->data) & 15))
		return pg_fail(ctx, PG_ERR_ARG, std::string(who) + ": data must be 16-byte aligned");
	return PG_OK;
}

static int hj_validate_proj(pg_ctx* ctx, const pg_col* proj, int nproj, uint32_t wR, uint32_t wS)
{
	if (nproj < 0 || nproj > HJ_MAX_COLS || (nproj && !proj))
		return pg_fail(ctx, PG_ERR_ARG, "join: 0..16 projected columns");
	for (int i = 0; i < nproj; ++i) {
		const pg_col& c = proj[i];
		uint32_t w = c.side ? wS : wR;
		if (c.side > 1 || (c.bytes != 4 && c.bytes != 8) || (c.off & 3) || c.off + c.bytes > w)
			return pg_fail(ctx, PG_ERR_UNSUPPORTED, "join: projected columns must be 4- or 8-byte, 4-byte aligned, inside the tuple");
	}
	return PG_OK;
}

// Build sides of 16-byte tuples whose key and build-projected columns lie in
// the tuple (one vector load per tuple).
static bool hj_vec16(const pg_rel* R, const HjBuildCols& bc)
{
	bool v = R->width == 16 && (R->key_off == 0 || R->key_off == 8) && R->key_bytes == 8 &&
		(reinterpret_cast<uintptr_t>(R->data) & 15) == 0;
	for (int c = 0; c < bc.n; ++c) v = v && bc.roff[c] + bc.words[c] <= 4;
	return v;
}

// Stream-ordered scratch freed when it goes out of scope (after the kernels
// queued on the stream that use it).
struct HjScratch {
	pg_ctx* ctx;
	cudaStream_t s;
	void* p = nullptr;
	HjScratch(pg_ctx* c, cudaStream_t st) : ctx(c), s(st) { }
	~HjScratch() { if (p) pg_free_async(ctx, s, p); }
	HjScratch(const HjScratch&) = delete;
	HjScratch& operator=(const HjScratch&) = delete;
};

// Partitioned probing of a hashed table (PG_TUNE_HASH_PARTITION = 2): the
// probe side is first partitioned on the top bits of its keys' hash
// (PG_FN_MIXRADIX), the same bits that place a key's home slot, into a scratch
// copy, so that each stretch of it looks up one 16 MB slice of the table; a
// table of packed values is built from R partitioned the same way. Rows come
// out in partition order (join output order is unspecified). Measured on the
// 16M x 256M sparse-key join it is slower (8.4 against 7.5 ms per step: the
// 256M-tuple partition pass costs more than the lookups save), so it is off
// unless asked for. Returns the number of partition bits, 0 for none.
static uint32_t hj_probe_partition_bits(const pg_ctx* ctx, const pg_hashtable* ht, uint64_t n)
{
	(void) n;
	if (ctx->tune[PG_TUNE_HASH_PARTITION] != 2 || ht->dense || ht->dense32 || !ht->slots || ht->log2cap < 12) return 0;
	const uint32_t lp = ht->log2cap > 20 ? ht->log2cap - 20 : 1;
	return std::min<uint32_t>(std::max<uint32_t>(lp, 1), 8);
}

// The table of R with host round trips: exact key and value ranges read back
// first, then a dense layout (duplicates counted and read back) or the hashed
// table. Fills the layout fields of `ht`.
static int hj_build_exact(pg_ctx* ctx, cudaStream_t s, const pg_rel* R, pg_hashtable* ht)
{
	int rc;
	ht->dense = false; ht->dense_val = nullptr; ht->dense_bits = nullptr; ht->dense32 = nullptr; ht->vmin = 0;
	ht->slots = nullptr; ht->side = nullptr; ht->nside = 0;
	if (R->n && ht->inline_val && ctx->tune[PG_TUNE_DENSE] != 2) {
		// Dense key domain (unique keys spanning at most 2|R| values, e.g. a
		// surrogate primary key 1..N): index by key - min, no hashing. Only
		// for packed values: the unique-key probe kernels read them inline.
		unsigned long long* mm = nullptr;
		if ((rc = pg_alloc_async(ctx, s, (void**) &mm, 64))) return rc;
		unsigned long long init[4] = {~0ull, 0, ~0ull, 0};
		PG_CUDA(ctx, cudaMemcpyAsync(mm, init, 32, cudaMemcpyHostToDevice, s));
		int blocks = (int) std::min<uint64_t>(pg_div_up(R->n, 256), (uint64_t) ctx->sm_count * 8);
		bool vec16 = R->width == 16 && (R->key_off == 0 || R->key_off == 8) && R->key_bytes == 8 &&
			(reinterpret_cast<uintptr_t>(R->data) & 15) == 0;
		for (int c = 0; c < ht->bcols.n; ++c) vec16 = vec16 && ht->bcols.roff[c] + ht->bcols.words[c] <= 4;
		const uint32_t kw = R->key_off / 4;
		const int vblocks = (int) std::min<uint64_t>(pg_div_up(R->n, 4 * 256), (uint64_t) ctx->sm_count * 8);
		if (vec16)
			k_key_minmax16<<<vblocks, 256, 0, s>>>((const uint4*) R->data, R->n, kw, ht->bcols, mm);
		else
			k_key_minmax<<<blocks, 256, 0, s>>>((const char*) R->data, R->n, R->width, R->key_off, R->key_bytes,
					ht->bcols, mm);
		PG_LAUNCHED(ctx);
		unsigned long long h[4];
		PG_CUDA(ctx, cudaMemcpyAsync(h, mm, 32, cudaMemcpyDeviceToHost, s));
		PG_CUDA(ctx, cudaStreamSynchronize(s));
		const long long kmin = (long long) (h[0] ^ (1ull << 63)), kmax = (long long) (h[1] ^ (1ull << 63));
		const unsigned long long range = (unsigned long long) kmax - (unsigned long long) kmin + 1;
		const bool narrow = h[3] - h[2] < 0xFFFFFFFFull;
		if (range != 0 && range <= std::max<uint64_t>(2 * R->n, 64) && range < (1ull << 34)) {
			int* dupflag_dev = reinterpret_cast<int*>(mm + 4);
			unsigned long long* present = mm + 5;
			PG_CUDA(ctx, cudaMemsetAsync(dupflag_dev, 0, 16, s));
			bool counted = false;
			if (narrow) {
				if ((rc = pg_alloc_async(ctx, s, (void**) &ht->dense32, range * 4))) return rc;
				PG_CUDA(ctx, cudaMemsetAsync(ht->dense32, 0xFF, range * 4, s));
				if (vec16) {
					// Plain stores; a duplicate key leaves fewer than |R| entries.
					k_dense32_store16<<<vblocks, 256, 0, s>>>((const uint4*) R->data, R->n, kw, ht->bcols, kmin, h[2],
							ht->dense32);
					PG_LAUNCHED(ctx);
					k_dense32_count<<<(int) std::min<uint64_t>(pg_div_up(range, 4 * 256), (uint64_t) ctx->sm_count * 8),
							256, 0, s>>>(ht->dense32, range, present);
					counted = true;
				} else {
					k_dense32_build<<<blocks, 256, 0, s>>>((const char*) R->data, R->n, R->width, R->key_off,
							R->key_bytes, ht->bcols, kmin, h[2], ht->dense32, dupflag_dev);
				}
			} else {
				const uint64_t words = pg_div_up(range, 32);
				if ((rc = pg_alloc_async(ctx, s, (void**) &ht->dense_val, range * 8))) return rc;
				if ((rc = pg_alloc_async(ctx, s, (void**) &ht->dense_bits, words * 4))) return rc;
				PG_CUDA(ctx, cudaMemsetAsync(ht->dense_bits, 0, words * 4, s));
				k_dense_build<<<blocks, 256, 0, s>>>((const char*) R->data, R->n, R->width, R->key_off,
						R->key_bytes, ht->bcols, ht->inline_val, kmin, ht->dense_val, ht->dense_bits, dupflag_dev);
			}
			PG_LAUNCHED(ctx);
			unsigned long long dh[2] = {0, 0};    // [dup flag word, present entries]
			PG_CUDA(ctx, cudaMemcpyAsync(dh, dupflag_dev, 16, cudaMemcpyDeviceToHost, s));
			PG_CUDA(ctx, cudaStreamSynchronize(s));
			const bool dup = counted ? dh[1] != R->n : (dh[0] & 0xFFFFFFFFull) != 0;
			if (!dup) {
				ht->dense = true; ht->unique = true; ht->dmin = kmin; ht->drange = range; ht->vmin = h[2]; ht->vmax = h[3];
				ht->vlo = h[2];
				ht->slots = nullptr; ht->side = nullptr; ht->nside = 0; ht->log2cap = 1; ht->capacity = 0;
				pg_free_async(ctx, s, mm);
				return PG_OK;
			}
			pg_free_async(ctx, s, ht->dense_val);
			pg_free_async(ctx, s, ht->dense_bits);
			pg_free_async(ctx, s, ht->dense32);
			ht->dense_val = nullptr; ht->dense_bits = nullptr; ht->dense32 = nullptr;
		}
		pg_free_async(ctx, s, mm);
	}
	uint64_t want = std::max<uint64_t>(1024, 2 * R->n);
	uint32_t lg = 10;
	while ((1ull << lg) < want) ++lg;
	ht->log2cap = lg; ht->capacity = 1ull << lg;
	ht->side_cap = HJ_SIDE_CAP0;
	if ((rc = pg_alloc_async(ctx, s, (void**) &ht->slots, ht->capacity * 16))) return rc;
	if ((rc = pg_alloc_async(ctx, s, (void**) &ht->side, ht->side_cap * 8 + 64))) return rc;
	// side buffer tail: [side_count u32][flags i32]
	unsigned int* side_count = reinterpret_cast<unsigned int*>(ht->side + ht->side_cap);
	int* flags = reinterpret_cast<int*>(side_count + 1);
	// Partitioned probing (hj_probe_partition_bits) of a table whose slots hold
	// the packed values (not row indices into R): the inserts run over a copy
	// of R partitioned on the keys' hash, filling one slice at a time.
	HjScratch part_buf(ctx, s);
	const char* Rb = (const char*) R->data;
	if (ht->inline_val && R->n >= (1ull << 20)) {
		if (const uint32_t lp = hj_probe_partition_bits(ctx, ht, ht->capacity)) {
			if ((rc = pg_alloc_async(ctx, s, &part_buf.p, R->n * R->width))) return rc;
			pg_hashfn f;
			f.fn = PG_FN_MIXRADIX; f.k = 0; f.min = 0; f.max = 0; f.bucketrange = 0;
			f.skipbits = 64 - lp; f.nbuckets = 1u << lp;
			if ((rc = pg_partition_fn(ctx, s, R, f, part_buf.p, nullptr))) return rc;
			Rb = (const char*) part_buf.p;
		}
	}
	for (int attempt = 0; attempt < 2; ++attempt) {
		PG_CUDA(ctx, cudaMemsetAsync(ht->slots, 0xFF, ht->capacity * 16, s));
		PG_CUDA(ctx, cudaMemsetAsync(side_count, 0, 8, s));
		if (R->n) {
			int blocks = (int) std::min<uint64_t>(pg_div_up(R->n, 256 * HT_ILP), (uint64_t) ctx->sm_count * 16);
			k_ht_build<<<blocks, 256, 0, s>>>(Rb, R->n, R->width, R->key_off, R->key_bytes,
					hj_pack_code(ht->bcols), ht->inline_val, ht->slots, ht->log2cap, ht->side, ht->side_cap,
					side_count, flags, ctx->d_status);
			PG_LAUNCHED(ctx);
		}
		unsigned int hdr[2];
		PG_CUDA(ctx, cudaMemcpyAsync(hdr, side_count, 8, cudaMemcpyDeviceToHost, s));
		if ((rc = pg_check_status(ctx, s, "pg_hashjoin_build"))) return rc;
		ht->nside = hdr[0];
		ht->unique = (hdr[1] & 1) == 0 && ht->nside <= 1;
		if (!(hdr[1] & 2)) break;
		// More empty-marker keys than the side list holds: grow it and rebuild.
		pg_free_async(ctx, s, ht->side);
		ht->side_cap = hdr[0];
		if ((rc = pg_alloc_async(ctx, s, (void**) &ht->side, ht->side_cap * 8 + 64))) return rc;
		side_count = reinterpret_cast<unsigned int*>(ht->side + ht->side_cap);
		flags = reinterpret_cast<int*>(side_count + 1);
	}
	return PG_OK;
}


// The narrow dense table of 16-byte tuples queued without host round trips
// (sample, fill, store, count); the header's checks are read by the probe
// kernels that take speculative tables, or by hj_settle.
static int hj_build_spec(pg_ctx* ctx, cudaStream_t s, const pg_rel* R, pg_hashtable* ht)
{
	int rc;
	const uint64_t cap = 2 * R->n + R->n / 8 + 4096;       // window entries the allocation holds
	ht->dense = true; ht->unique = true;
	ht->slots = nullptr; ht->side = nullptr; ht->nside = 0; ht->log2cap = 1; ht->capacity = 0;
	ht->dense_val = nullptr; ht->dense_bits = nullptr;
	ht->hdr = nullptr; ht->dense32_base = nullptr; ht->dense32 = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &ht->hdr, sizeof(HjDenseHdr)))) return rc;
	if ((rc = pg_alloc_async(ctx, s, (void**) &ht->dense32_base, cap * 4))) return rc;
	ht->dense32 = ht->dense32_base;
	ht->dmin = 0; ht->drange = cap; ht->vmin = 0; ht->vlo = 0; ht->vmax = 0;     // bounds until settled
	const uint32_t kw = R->key_off / 4;
	const uint32_t pk = hj_pack16_code(ht->bcols);
	k_dense_prep16<<<1, 1024, 0, s>>>((const uint4*) R->data, R->n, kw, pk, cap, ht->hdr);
	PG_LAUNCHED(ctx);
	const int fgrid = (int) std::min<uint64_t>(pg_div_up(cap / 4 + 1, 256), (uint64_t) ctx->sm_count * 8);
	k_dense_fill16<<<fgrid, 256, 0, s>>>(ht->dense32_base, ht->hdr);
	PG_LAUNCHED(ctx);
	const int sgrid = (int) std::min<uint64_t>(pg_div_up(R->n, 4 * 256), (uint64_t) ctx->sm_count * 16);
	k_dense32_spec16<<<sgrid, 256, 0, s>>>((const uint4*) R->data, R->n, kw, pk, ht->dense32_base, ht->hdr);
	PG_LAUNCHED(ctx);
	k_dense32_count_spec<<<fgrid, 256, 0, s>>>(ht->dense32_base, ht->hdr);
	PG_LAUNCHED(ctx);
	// Probes on other streams wait for these kernels (the build returns
	// without synchronising).
	PG_CUDA(ctx, cudaEventCreateWithFlags(&ht->built, cudaEventDisableTiming));
	PG_CUDA(ctx, cudaEventRecord(ht->built, s));
	ht->spec.store(true, std::memory_order_release);
	return PG_OK;
}

static bool hj_hdr_ok(const HjDenseHdr& h)
{
	return h.flags == 0 && h.present == h.n;
}

int hj_settle(pg_ctx* ctx, pg_hashtable* ht)
{
	if (!ht || !ht->spec.load(std::memory_order_acquire)) return PG_OK;
	std::lock_guard<std::mutex> g(ht->mu);
	if (!ht->spec.load(std::memory_order_relaxed)) return PG_OK;
	cudaStream_t s = ht->stream;
	HjDenseHdr h;
	PG_CUDA(ctx, cudaMemcpyAsync(&h, ht->hdr, sizeof h, cudaMemcpyDeviceToHost, s));
	PG_CUDA(ctx, cudaStreamSynchronize(s));
	if (hj_hdr_ok(h)) {
		// Exact layout, as hj_build_exact would have made it: the window
		// narrowed to the keys present, entries based on the smallest value.
		const long long kmin = (long long) (h.kmin ^ (1ull << 63)), kmax = (long long) (h.kmax ^ (1ull << 63));
		const unsigned long long off = (unsigned long long) kmin - (unsigned long long) h.dmin;
		uint32_t* win = ht->dense32_base + off;
		const unsigned long long range = (unsigned long long) kmax - (unsigned long long) kmin + 1;
		// A copy too when the narrowed window would not start on a 16-byte
		// boundary: table readers (the image checksum's 8-byte words, vector
		// loads) rely on the alignment of an allocation.
		if (h.vlo != h.vmin || (off & 3) != 0) {
			int rc;
			if ((rc = pg_alloc_async(ctx, s, (void**) &ht->dense32_copy, range * 4))) return rc;
			const int grid = (int) std::min<uint64_t>(pg_div_up(range, 256), (uint64_t) ctx->sm_count * 8);
			k_dense32_rebase<<<grid, 256, 0, s>>>(win, ht->dense32_copy, range, (uint32_t) (h.vlo - h.vmin));
			PG_LAUNCHED(ctx);
			PG_CUDA(ctx, cudaStreamSynchronize(s));      // users on other streams read the copy next
			win = ht->dense32_copy;
		}
		ht->dense32 = win;
		ht->dmin = kmin;
		ht->drange = range;
		ht->vmin = h.vlo; ht->vlo = h.vlo; ht->vmax = h.vhi;
		ht->spec.store(false, std::memory_order_release);
		return PG_OK;
	}
	// Refuted (a repeated key, a key or value the sample missed): rebuild
	// from the build relation with the exact ranges. Probes queued with the
	// header see it refuted and touch no entry, so the window can go.
	pg_free_async(ctx, s, ht->dense32_base);
	ht->dense32_base = nullptr; ht->dense32 = nullptr;
	int rc = hj_build_exact(ctx, s, &ht->rel, ht);
	ht->spec.store(false, std::memory_order_release);
	return rc;
}

extern "C" int pg_hashjoin_build(pg_ctx* ctx, pg_stream stream, const pg_rel* R,
		const pg_col* proj, int nproj, pg_hashtable** out)
{
	if (!ctx || !out) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_build: null argument");
	int rc;
	if ((rc = hj_validate_rel(ctx, R, "pg_hashjoin_build"))) return rc;
	if ((rc = hj_validate_proj(ctx, proj, nproj, R->width, 1u << 30))) return rc;
	cudaStream_t s = (cudaStream_t) stream;
	pg_hashtable* ht = new pg_hashtable();
	ht->nbuild = R->n; ht->R = (const char*) R->data; ht->wR = R->width; ht->bkey_bytes = R->key_bytes;
	ht->nproj = nproj;
	ht->stream = s;
	for (int i = 0; i < nproj; ++i) ht->proj[i] = proj[i];
	uint32_t bbytes = 0;
	ht->bcols.n = 0;
	for (int i = 0; i < nproj; ++i)
		if (proj[i].side == 0) {
			ht->bcols.roff[ht->bcols.n] = (uint16_t) (proj[i].off / 4);
			ht->bcols.words[ht->bcols.n] = (uint8_t) (proj[i].bytes / 4);
			ht->bcols.n++;
			bbytes += proj[i].bytes;
		}
	ht->inline_val = bbytes <= 8;
	ht->rel = *R;
	ht->spec.store(false); ht->hdr = nullptr; ht->dense32_base = nullptr; ht->dense32_copy = nullptr;
	ht->built = nullptr;
	const int64_t spec = ctx->tune[PG_TUNE_BUILD_SPEC];
	if (R->n && ht->inline_val && ctx->tune[PG_TUNE_DENSE] != 2 && spec != 2 && hj_vec16(R, ht->bcols) &&
			(spec == 1 || R->n >= HJ_SPEC_MIN_TUPLES))
		rc = hj_build_spec(ctx, s, R, ht);
	else
		rc = hj_build_exact(ctx, s, R, ht);
	if (rc) { pg_hashtable_free(ctx, ht); return rc; }
	*out = ht;
	return PG_OK;
}

extern "C" int pg_hashtable_free(pg_ctx* ctx, pg_hashtable* ht)
{
	if (!ht) return PG_OK;
	// Probes finish before they return (they read their counts back), so
	// only work still queued on the build stream can use the table.
	cudaStreamSynchronize(ht->stream);
	pg_free_async(ctx, ht->stream, ht->slots);
	pg_free_async(ctx, ht->stream, ht->side);
	pg_free_async(ctx, ht->stream, ht->dense_val);
	pg_free_async(ctx, ht->stream, ht->dense_bits);
	if (ht->dense32_base || ht->dense32_copy) {
		pg_free_async(ctx, ht->stream, ht->dense32_base);
		pg_free_async(ctx, ht->stream, ht->dense32_copy);
	} else {
		pg_free_async(ctx, ht->stream, ht->dense32);
	}
	pg_free_async(ctx, ht->stream, ht->hdr);
	if (ht->built) cudaEventDestroy(ht->built);
	delete ht;
	return PG_OK;
}

static int hj_make_cols(pg_ctx* ctx, const pg_hashtable* ht, const pg_col* proj, int nproj, HjCols* pc)
{
	if (nproj != ht->nproj) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_probe: projection differs from the build's");
	pc->n = nproj;
	int ow = 0, boff = 0;
	for (int i = 0; i < nproj; ++i) {
		if (proj[i].side != ht->proj[i].side || (proj[i].side == 0 &&
				(proj[i].off != ht->proj[i].off || proj[i].bytes != ht->proj[i].bytes)))
			return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_probe: projection differs from the build's");
		pc->side[i] = (uint8_t) proj[i].side;
		pc->words[i] = (uint8_t) (proj[i].bytes / 4);
		if (proj[i].side) pc->src[i] = (uint16_t) (proj[i].off / 4);
		else if (ht->inline_val) { pc->src[i] = (uint16_t) boff; boff += proj[i].bytes / 4; }
		else pc->src[i] = (uint16_t) (proj[i].off / 4);
		ow += pc->words[i];
	}
	pc->ow_words = ow;
	return PG_OK;
}

// Internal results of the probe launch on a speculative table (never returned
// through the C ABI): the chosen kernel needs the settled table, or the
// build's checks failed and the probe wrote nothing.
#define HJ_NEED_SETTLE 1001
#define HJ_SPEC_REFUTED 1002

#define HJ_TWO_PASS_MIN_BYTES (56ull << 20)   // dense tables above this probe in two passes
#define HJ_TWO_PASS_MAX_BYTES (112ull << 20)  // ... up to this (half must fit in L2)

// Launches the unique-key probe over n tuples at S (device) into `out`;
// counts/sums accumulate in acc[1..2], the output cursor is acc[0].
// With `counts` (device, one word per 256-tuple chunk) and cap >= n, 16-byte
// probes use the warp-independent kernel and write rows positionally; the
// caller then compacts when fewer than n rows matched (*positional = true).
// The staged probe over n tuples: a persistent grid of as many CTAs per SM as
// the tile buffers allow.
template <bool M, int D, int I>
static int hjg_launch(pg_ctx* ctx, cudaStream_t s, const char* S, uint64_t n, uint32_t W, uint32_t koff,
		uint32_t kbytes, const HjProbeTable& tb, const HjWordMap& wm, char* out, uint64_t cap,
		unsigned long long* acc)
{
	const uint32_t T = HJG_THREADS * I;
	const int smem = (int) (HJG_BUFS * T * W + T * (8 + 2));
	PG_CUDA(ctx, cudaFuncSetAttribute(k_probe_staged<M, D, I>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
	int per_sm = 0;
	PG_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_probe_staged<M, D, I>, HJG_THREADS, smem));
	const int grid = (int) std::min<uint64_t>(pg_div_up(n, T), (uint64_t) ctx->sm_count * std::max(per_sm, 1));
	k_probe_staged<M, D, I><<<grid, HJG_THREADS, smem, s>>>(S, n, W, koff, kbytes, tb, wm, M ? out : nullptr,
			M ? cap : 0, acc, acc + 1, ctx->d_status);
	PG_LAUNCHED(ctx);
	return PG_OK;
}

static int hj_launch_unique(pg_ctx* ctx, cudaStream_t s, const pg_hashtable* ht, const char* S,
		uint64_t n, uint32_t W, uint32_t koff, uint32_t kbytes, const HjCols& pc, char* out,
		uint64_t cap, unsigned long long* acc, bool materialize, int sum_col,
		uint64_t* counts = nullptr, bool* positional = nullptr, const PgPred16* pred = nullptr)
{
	if (positional) *positional = false;
	const uint64_t ntiles = pg_div_up(n, HJ_TILE);
	HjProbeTable tb;
	// A speculative table is described by its header and window base alone
	// (read once: another thread may settle it meanwhile).
	const bool spec = ht->spec.load(std::memory_order_acquire);
	if (spec) {
		tb = HjProbeTable();
		tb.hdr = ht->hdr; tb.dense32 = ht->dense32_base;
	} else {
		tb.slots = ht->slots; tb.log2cap = ht->log2cap; tb.side = ht->side; tb.nside = ht->nside;
		tb.dense_val = ht->dense_val; tb.dense_bits = ht->dense_bits; tb.dmin = ht->dmin; tb.drange = ht->drange;
		tb.dense32 = ht->dense32; tb.vmin = ht->vmin;
		tb.hdr = nullptr;
	}
	// Built-in table-load policy: evict-last for half of the table's lines
	// and lookups kept in L1 (measured on the 16M x 256M join: 2.19 against
	// 2.32 ms per step uniform, 1.88 against 2.52 ms with Zipf s=1.0 probes,
	// whose hot entries L1 serves instead of one L2 slice).
	const int64_t ck = ctx->tune[PG_TUNE_PROBE_CACHE];
	tb.cache = ck ? (uint32_t) (ck & 255) : (4u << 4) | 128u;
	const int mode = spec ? 2 : ht->dense ? (ht->dense32 ? 2 : 1) : 0;
	const bool fast16 = W == 16 && (koff == 0 || koff == 8) && kbytes == 8 && pc.ow_words == 4 &&
		(reinterpret_cast<uintptr_t>(S) & 15) == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0;
	if (pred && !fast16)
		return pg_fail(ctx, PG_ERR_UNSUPPORTED, "join probe: predicates need 16-byte probe tuples and output rows");
	if (fast16) {
		const int smem = 3 * HJT_TILE * 16;
		uint32_t wsel = 0, o = 0, sum_w0 = 0, sum_words = 0;
		for (int c = 0; c < pc.n; ++c) {
			if (c == sum_col) { sum_w0 = o; sum_words = pc.words[c]; }
			for (int q = 0; q < pc.words[c]; ++q, ++o)
				wsel |= (pc.side[c] ? (pc.src[c] + q) : (4u + pc.src[c] + q)) << (4 * o);
		}
		// Predicates run in the register-loading dense kernels only.
		if (pred && (mode == 0 || (materialize && !(counts && cap >= n))))
			return pg_fail(ctx, PG_ERR_UNSUPPORTED, "join probe: predicates need a dense table and room for every probe row");
		const bool tiled = !pred && ctx->tune[PG_TUNE_PROBE_VARIANT] == 2;
		if (!materialize || (counts && cap >= n && !tiled)) {
			// Lookups in flight per lane: 8 for dense tables when asked, else 4.
			const int items = (mode != 0 && ctx->tune[PG_TUNE_PROBE_ITEMS] == 8) ? 8 : 4;
			const int psmem = PW_WARPS * PW_STAGES * 32 * items * 16;
			// Persistent grid: CTAs per SM from the tuning table, else as many
			// as the shared memory holds for dense tables (4 at 4 items, 3 at
			// 8: more resident warps evict table lines from L2 faster than
			// they hide latency) and 2 for hashed ones.
			const int64_t per_sm = ctx->tune[PG_TUNE_PROBE_CTAS_PER_SM] > 0
				? std::min<int64_t>(items > 4 ? 3 : 5, ctx->tune[PG_TUNE_PROBE_CTAS_PER_SM])
				: (mode != 0 ? (items > 4 ? 3 : 4) : 2);
			const int pgrid = (int) std::min<uint64_t>(pg_div_up(pg_div_up(n, 32 * items), PW_WARPS),
					(uint64_t) ctx->sm_count * per_sm);
			// Two passes over half the table each when the dense table is
			// larger than L2 keeps next to the streams (knob: 1 one pass,
			// 2 two passes, 0 by table size).
			const uint64_t tbytes = mode == 2 ? ht->drange * 4 : ht->drange * 8;
			const int64_t pk = pred ? 1 : ctx->tune[PG_TUNE_PROBE_PASSES];
			// Dense tables take the register-loading probe unless the knob asks
			// for the staged one (1) or the non-prefetching one (4).
			const int64_t var = pred ? 0 : ctx->tune[PG_TUNE_PROBE_VARIANT];
			const bool direct = mode != 0 && (var == 0 || var == 3 || var == 4 || var == 5);
			const int passes = mode == 0 || pk == 1 ? 1
				: (pk == 2 || (!direct && tbytes > HJ_TWO_PASS_MIN_BYTES && tbytes <= HJ_TWO_PASS_MAX_BYTES)) ? 2 : 1;
			const uint64_t dr = mode == 0 ? 0 : ht->drange;
			// Only the register-loading dense kernels read a speculative
			// table's window from its header.
			if (spec && (!direct || pred || passes != 1)) return HJ_NEED_SETTLE;
			for (int pass = 0; pass < passes; ++pass) {
				const int run = passes == 1 ? -1 : pass;
				const uint64_t dlo = passes == 1 ? 0 : (pass == 0 ? 0 : dr / 2);
				const uint64_t dhi = passes == 1 ? dr : (pass == 0 ? dr / 2 : dr);
				if (direct) {
					// Grids of several waves (4 CTAs of 8 warps resident per SM):
					// 24 CTAs per SM with prefetch, 80 without, measured best on
					// the 16M x 256M join; each warp adds its count once.
					const uint64_t wchunks = pg_div_up(pg_div_up(n, PW_CHUNK), PW_WARPS);
					const bool pf = var != 4;
					const int64_t want = ctx->tune[PG_TUNE_PROBE_CTAS_PER_SM] > 0
						? std::min<int64_t>(1 << 14, ctx->tune[PG_TUNE_PROBE_CTAS_PER_SM]) : (pf ? 24 : 80);
					const int dgrid = (int) std::min<uint64_t>(wchunks, (uint64_t) ctx->sm_count * want);
#define PD_LAUNCH(M, D, P) k_probe16_direct<M, D, P><<<dgrid, PW_WARPS * 32, 0, s>>>(S, n, koff, tb, wsel, sum_w0, \
						sum_words, M ? out : nullptr, M ? counts : nullptr, M ? acc : acc + 1, M ? -1 : sum_col, dlo, dhi, run)
					// The standard (P$1, B$1) rows of a narrow dense table take the
					// deeper pipeline by default (72 CTAs per SM in waves, 4 resident
					// at 64 registers: measured best on the 16M x 256M join);
					// variant 3 selects the one-chunk-prefetch kernel.
					const int g5 = (int) std::min<uint64_t>(wchunks, (uint64_t) ctx->sm_count *
							(ctx->tune[PG_TUNE_PROBE_CTAS_PER_SM] > 0 ? ctx->tune[PG_TUNE_PROBE_CTAS_PER_SM] : 72));
					if (pred) {
						const PgPred16 pr = *pred;
						if (materialize && mode == 2) {
							// Compacting pipeline: rows land compact, nothing to move after.
							const int ssmem = PW_WARPS * HJ_STAGE_ROWS * 16;
							if (wsel == 0x5432u) {
								PG_CUDA(ctx, cudaFuncSetAttribute(k_probe16_stage<true, true>,
										cudaFuncAttributeMaxDynamicSharedMemorySize, ssmem));
								k_probe16_stage<true, true><<<g5, PW_WARPS * 32, ssmem, s>>>(S, n, koff, tb, wsel, out,
										cap, acc, pr);
							} else {
								PG_CUDA(ctx, cudaFuncSetAttribute(k_probe16_stage<true, false>,
										cudaFuncAttributeMaxDynamicSharedMemorySize, ssmem));
								k_probe16_stage<true, false><<<g5, PW_WARPS * 32, ssmem, s>>>(S, n, koff, tb, wsel, out,
										cap, acc, pr);
							}
							PG_LAUNCHED(ctx);
							return PG_OK;
						} else if (materialize && mode == 2)
							k_probe16_direct<true, 2, true, false, true><<<dgrid, PW_WARPS * 32, 0, s>>>(S, n, koff, tb,
									wsel, sum_w0, sum_words, out, counts, acc, -1, dlo, dhi, run, pr);
						else if (materialize)
							k_probe16_direct<true, 1, true, false, true><<<dgrid, PW_WARPS * 32, 0, s>>>(S, n, koff, tb,
									wsel, sum_w0, sum_words, out, counts, acc, -1, dlo, dhi, run, pr);
						else if (mode == 2)
							k_probe16_direct<false, 2, true, false, true><<<dgrid, PW_WARPS * 32, 0, s>>>(S, n, koff, tb,
									wsel, sum_w0, sum_words, nullptr, nullptr, acc + 1, sum_col, dlo, dhi, run, pr);
						else
							k_probe16_direct<false, 1, true, false, true><<<dgrid, PW_WARPS * 32, 0, s>>>(S, n, koff, tb,
									wsel, sum_w0, sum_words, nullptr, nullptr, acc + 1, sum_col, dlo, dhi, run, pr);
					} else if (materialize && mode == 2 && (var == 0 || var == 5) && wsel == 0x5432u && passes == 1) {
						k_probe16_deep<false><<<g5, PW_WARPS * 32, 0, s>>>(S, n, koff, tb, out, counts, acc, PgPred16());
					} else if (materialize && mode == 2 && pf && wsel == 0x5432u) {
						k_probe16_direct<true, 2, true, true><<<dgrid, PW_WARPS * 32, 0, s>>>(S, n, koff, tb, wsel, sum_w0,
								sum_words, out, counts, acc, -1, dlo, dhi, run);
					} else if (materialize) {
						if (mode == 2) { if (pf) PD_LAUNCH(true, 2, true); else PD_LAUNCH(true, 2, false); }
						else { if (pf) PD_LAUNCH(true, 1, true); else PD_LAUNCH(true, 1, false); }
					} else {
						if (mode == 2) { if (pf) PD_LAUNCH(false, 2, true); else PD_LAUNCH(false, 2, false); }
						else { if (pf) PD_LAUNCH(false, 1, true); else PD_LAUNCH(false, 1, false); }
					}
#undef PD_LAUNCH
					PG_LAUNCHED(ctx);
					continue;
				}
#define PW_LAUNCH(M, D, I) do { \
				PG_CUDA(ctx, cudaFuncSetAttribute(k_probe16_warp<M, D, I>, cudaFuncAttributeMaxDynamicSharedMemorySize, psmem)); \
				k_probe16_warp<M, D, I><<<pgrid, PW_WARPS * 32, psmem, s>>>(S, n, koff, tb, wsel, sum_w0, sum_words, \
						M ? out : nullptr, M ? counts : nullptr, M ? acc : acc + 1, M ? -1 : sum_col, ctx->d_status, \
						dlo, dhi, run); } while (0)
				if (materialize) {
					if (mode == 2) { if (items == 8) PW_LAUNCH(true, 2, 8); else PW_LAUNCH(true, 2, 4); }
					else if (mode == 1) { if (items == 8) PW_LAUNCH(true, 1, 8); else PW_LAUNCH(true, 1, 4); }
					else PW_LAUNCH(true, 0, 4);
				} else {
					if (mode == 2) { if (items == 8) PW_LAUNCH(false, 2, 8); else PW_LAUNCH(false, 2, 4); }
					else if (mode == 1) { if (items == 8) PW_LAUNCH(false, 1, 8); else PW_LAUNCH(false, 1, 4); }
					else PW_LAUNCH(false, 0, 4);
				}
#undef PW_LAUNCH
				PG_LAUNCHED(ctx);
			}
			if (positional) *positional = materialize;
			return PG_OK;
		}
		if (spec) return HJ_NEED_SETTLE;
		const int grid = (int) std::min<uint64_t>(pg_div_up(n, HJT_TILE), (uint64_t) ctx->sm_count * 3);
#define HJT_LAUNCH(M, D) do { \
			PG_CUDA(ctx, cudaFuncSetAttribute(k_probe16_tma<M, D>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem)); \
			k_probe16_tma<M, D><<<grid, HJT_THREADS, smem, s>>>(S, n, koff, tb, wsel, sum_w0, sum_words, \
					M ? out : nullptr, M ? cap : 0, acc, acc + 1, M ? -1 : sum_col, ctx->d_status); } while (0)
		if (materialize) { if (mode == 2) HJT_LAUNCH(true, 2); else if (mode == 1) HJT_LAUNCH(true, 1); else HJT_LAUNCH(true, 0); }
		else { if (mode == 2) HJT_LAUNCH(false, 2); else if (mode == 1) HJT_LAUNCH(false, 1); else HJT_LAUNCH(false, 0); }
#undef HJT_LAUNCH
		PG_LAUNCHED(ctx);
		return PG_OK;
	}
	// Other widths: materialised rows from dense tables are staged through
	// shared memory when tuples and rows are whole words and a tile fits the
	// buffers. Counts and sums, which write nothing, read their key and sum
	// words per thread (0.44 against 0.51 ms staged on 64M 24-byte tuples), and
	// so do hashed tables, whose pending bucket loads cost the staged kernel
	// registers (2.34 against 2.40 ms).
	if (spec) return HJ_NEED_SETTLE;
	const int64_t wide = ctx->tune[PG_TUNE_PROBE_WIDE];
	const bool staged = wide == 2 || wide == 3 || (wide == 0 && materialize && mode != 0);
	if (staged && W % 4 == 0 && W <= HJG_MAX_W && koff % 4 == 0 && pc.ow_words >= 1 &&
			pc.ow_words <= HJG_MAX_OW && (reinterpret_cast<uintptr_t>(S) & 15) == 0 &&
			(!materialize || (reinterpret_cast<uintptr_t>(out) & 3) == 0)) {
		HjWordMap wm = {};
		uint32_t o = 0;
		for (int c = 0; c < pc.n; ++c) {
			if (c == sum_col) { wm.sum_w0 = o; wm.sum_words = pc.words[c]; }
			for (int q = 0; q < pc.words[c]; ++q, ++o)
				wm.src[o] = (uint8_t) (pc.side[c] ? pc.src[c] + q : 64 + pc.src[c] + q);
		}
		wm.ow = o;
		wm.uw = (o % 2 == 0 && (reinterpret_cast<uintptr_t>(out) & 7) == 0) ? 2 : 1;
		const bool four = wide == 2;
#define HJG_GO(M, D) (four ? hjg_launch<M, D, 4>(ctx, s, S, n, W, koff, kbytes, tb, wm, out, cap, acc) \
		: hjg_launch<M, D, 2>(ctx, s, S, n, W, koff, kbytes, tb, wm, out, cap, acc))
		if (materialize) return mode == 2 ? HJG_GO(true, 2) : mode == 1 ? HJG_GO(true, 1) : HJG_GO(true, 0);
		return mode == 2 ? HJG_GO(false, 2) : mode == 1 ? HJG_GO(false, 1) : HJG_GO(false, 0);
#undef HJG_GO
	}
	const int grid = (int) std::min<uint64_t>(ntiles, (uint64_t) ctx->sm_count * 8);
	if (materialize)
		k_probe_unique<true, false><<<grid, HJ_THREADS, 0, s>>>(S, n, W, koff, kbytes, tb, ht->dense,
				pc, out, cap, acc, acc + 1, -1, ctx->d_status);
	else
		k_probe_unique<false, false><<<grid, HJ_THREADS, 0, s>>>(S, n, W, koff, kbytes, tb, ht->dense,
				pc, nullptr, 0, acc, acc + 1, sum_col, ctx->d_status);
	PG_LAUNCHED(ctx);
	return PG_OK;
}

// Compacts a positional probe output of n tuples with `total` matches in place
// (through a scratch copy): chunk counts are scanned into offsets first.
static int hj_compact(pg_ctx* ctx, cudaStream_t s, char* out, uint64_t n, uint64_t* counts, uint64_t total)
{
	const uint64_t nchunks = pg_div_up(n, PW_CHUNK);
	int rc;
	uint64_t* offs = nullptr;
	char* tmp = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &offs, nchunks * 8))) return rc;
	if ((rc = pg_alloc_async(ctx, s, (void**) &tmp, std::max<uint64_t>(total, 1) * 16))) return rc;
	k_chunk_totals<<<(int) std::min<uint64_t>(pg_div_up(nchunks, 256), (uint64_t) ctx->sm_count * 8), 256, 0, s>>>(
			counts, offs, nchunks, n);
	PG_LAUNCHED(ctx);
	if ((rc = pg_scan_u64(ctx, s, offs, nchunks, nullptr))) return rc;
	const int grid = (int) std::min<uint64_t>(nchunks, (uint64_t) ctx->sm_count * 16);
	k_compact_chunks<<<grid, 256, 0, s>>>(reinterpret_cast<const uint4*>(out), counts, offs, nchunks, n,
			reinterpret_cast<uint4*>(tmp), total);
	PG_LAUNCHED(ctx);
	if (total) PG_CUDA(ctx, cudaMemcpyAsync(out, tmp, total * 16, cudaMemcpyDeviceToDevice, s));
	pg_free_async(ctx, s, offs);
	pg_free_async(ctx, s, tmp);
	return PG_OK;
}

// The probe's accumulators acc[0..3] with, in acc[4..7], a speculative
// table's checks (flags, present entries, tuples) and the context's status
// word, so that one copy brings all of them back.
__global__ void k_probe_tail(unsigned long long* __restrict__ acc, const HjDenseHdr* __restrict__ hdr,
		const int* __restrict__ status)
{
	acc[4] = hdr ? (unsigned long long) (unsigned) hdr->flags : 0;
	acc[5] = hdr ? hdr->present : 0;
	acc[6] = hdr ? hdr->n : 0;
	acc[7] = (unsigned long long) (unsigned) *status;
}

// One round trip after a probe: h = acc[0..7]; a non-zero status fails the
// call; *refuted: the speculative table's checks failed (nothing was probed).
static int hj_readback(pg_ctx* ctx, cudaStream_t s, unsigned long long* acc, const HjDenseHdr* hdr,
		unsigned long long (&h)[8], bool* refuted, const char* what)
{
	k_probe_tail<<<1, 1, 0, s>>>(acc, hdr, ctx->d_status);
	PG_LAUNCHED(ctx);
	PG_CUDA(ctx, cudaMemcpyAsync(h, acc, sizeof h, cudaMemcpyDeviceToHost, s));
	PG_CUDA(ctx, cudaStreamSynchronize(s));
	if (h[7]) return pg_status_fail(ctx, s, (int) h[7], what);
	*refuted = hdr && !(h[4] == 0 && h[5] == h[6]);
	return PG_OK;
}

// pg_hashjoin_probe; with `pred`, the probe tuples failing it take no part
// (only for the dense 16-byte layouts the register-loading kernels handle).
static int hj_probe_run(pg_ctx* ctx, pg_stream stream, pg_hashtable* ht,
		const pg_rel* S_in, const pg_col* proj, int nproj,
		void* out, uint64_t out_capacity, int flags, int sum_col, pg_join_result* res, const PgPred16* pred)
{
	if (!ctx || !ht || !res) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_probe: null argument");
	int rc;
	if ((rc = hj_validate_rel(ctx, S_in, "pg_hashjoin_probe"))) return rc;
	if ((rc = hj_validate_proj(ctx, proj, nproj, ht->wR, S_in->width))) return rc;
	HjCols pc;
	if ((rc = hj_make_cols(ctx, ht, proj, nproj, &pc))) return rc;
	const bool materialize = (flags & PG_JOIN_MATERIALIZE) != 0;
	if (sum_col >= nproj) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_probe: sum_col out of range");
	if (!(flags & PG_JOIN_SUM)) sum_col = -1;
	if (materialize && out_capacity && !out) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_probe: null output");
	cudaStream_t s = (cudaStream_t) stream;
	res->n_out = 0; res->sum = 0;
	if (S_in->n == 0) return PG_OK;
	pg_rel Sloc = *S_in;
	const pg_rel* S = &Sloc;
	HjScratch part_buf(ctx, s);
	if (const uint32_t lp = hj_probe_partition_bits(ctx, ht, S_in->n)) {
		if ((rc = pg_alloc_async(ctx, s, &part_buf.p, S_in->n * S_in->width))) return rc;
		pg_hashfn f;
		f.fn = PG_FN_MIXRADIX; f.k = 0; f.min = 0; f.max = 0; f.bucketrange = 0;
		f.skipbits = 64 - lp; f.nbuckets = 1u << lp;
		if ((rc = pg_partition_fn(ctx, s, S_in, f, part_buf.p, nullptr))) return rc;
		Sloc.data = part_buf.p;
	}
	unsigned long long* acc = nullptr;   // [cursor, count, sum, spare]
	if ((rc = pg_alloc_async(ctx, s, (void**) &acc, 64))) return rc;
	PG_CUDA(ctx, cudaMemsetAsync(acc, 0, 64, s));
	const uint64_t ntiles = pg_div_up(S->n, HJ_TILE);
	unsigned long long host_acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};

	if (ht->unique && ht->inline_val) {
		const char* Sd = (const char*) S->data;
		// A speculative table's checks come back with the counts; when they
		// failed, the kernels wrote nothing and the caller rebuilds.
		const bool spec = ht->spec.load(std::memory_order_acquire);
		const HjDenseHdr* hdr = spec ? ht->hdr : nullptr;
		bool refuted = false;
		if (spec) PG_CUDA(ctx, cudaStreamWaitEvent(s, ht->built, 0));
		if (materialize) {
			uint64_t* counts = nullptr;
			bool positional = false;
			if ((rc = pg_alloc_async(ctx, s, (void**) &counts, pg_div_up(S->n, PW_CHUNK) * 8))) return rc;
			if ((rc = hj_launch_unique(ctx, s, ht, Sd, S->n, S->width, S->key_off, S->key_bytes, pc,
					(char*) out, out_capacity, acc, true, -1, counts, &positional, pred))) {
				pg_free_async(ctx, s, counts); pg_free_async(ctx, s, acc);
				return rc;
			}
			if ((rc = hj_readback(ctx, s, acc, hdr, host_acc, &refuted, "pg_hashjoin_probe"))) return rc;
			if (refuted) {
				pg_free_async(ctx, s, counts); pg_free_async(ctx, s, acc);
				return HJ_SPEC_REFUTED;
			}
			res->n_out = host_acc[0];
			if (positional && res->n_out < S->n) {
				if ((rc = hj_compact(ctx, s, (char*) out, S->n, counts, res->n_out))) return rc;
				if ((rc = pg_check_status(ctx, s, "pg_hashjoin_probe"))) return rc;
			}
			pg_free_async(ctx, s, counts);
			if (sum_col >= 0 || (flags & PG_JOIN_COUNT)) {
				// Fold count/sum with a second, non-materialising pass.
				if ((rc = hj_launch_unique(ctx, s, ht, Sd, S->n, S->width, S->key_off, S->key_bytes, pc,
						nullptr, 0, acc, false, sum_col, nullptr, nullptr, pred))) return rc;
				PG_CUDA(ctx, cudaMemcpyAsync(host_acc, acc, 32, cudaMemcpyDeviceToHost, s));
				if ((rc = pg_check_status(ctx, s, "pg_hashjoin_probe"))) return rc;
				res->sum = (int64_t) host_acc[2];
			}
		} else {
			if ((rc = hj_launch_unique(ctx, s, ht, Sd, S->n, S->width, S->key_off, S->key_bytes, pc,
					nullptr, 0, acc, false, sum_col, nullptr, nullptr, pred))) {
				pg_free_async(ctx, s, acc);
				return rc;
			}
			if ((rc = hj_readback(ctx, s, acc, hdr, host_acc, &refuted, "pg_hashjoin_probe"))) return rc;
			if (refuted) {
				pg_free_async(ctx, s, acc);
				return HJ_SPEC_REFUTED;
			}
			res->n_out = host_acc[1];
			res->sum = (int64_t) host_acc[2];
		}
		pg_free_async(ctx, s, acc);
		if (materialize && res->n_out > out_capacity)
			return pg_fail(ctx, PG_ERR_OUTPUT_FULL, "pg_hashjoin_probe: output capacity too small");
		return PG_OK;
	}

	// General path: one CTA per tile for the count pass, scan, write pass.
	// It walks hashed slots, which a dense table does not have.
	if (ht->dense) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_probe: dense table on the general path");
	uint64_t* tile_counts = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &tile_counts, (ntiles + 1) * 8))) return rc;
	k_probe_general<false><<<(unsigned) ntiles, HJ_THREADS, 0, s>>>((const char*) S->data, S->n, S->width,
			S->key_off, S->key_bytes, ht->slots, ht->log2cap, ht->side, ht->nside, pc, ht->inline_val,
			ht->R, ht->wR, tile_counts, nullptr, acc + 1, sum_col, ctx->d_status);
	PG_LAUNCHED(ctx);
	if ((rc = pg_scan_u64(ctx, s, tile_counts, ntiles, (uint64_t*) acc))) return rc;
	PG_CUDA(ctx, cudaMemcpyAsync(host_acc, acc, 32, cudaMemcpyDeviceToHost, s));
	if ((rc = pg_check_status(ctx, s, "pg_hashjoin_probe"))) return rc;
	res->n_out = host_acc[0];
	res->sum = (int64_t) host_acc[2];
	if (materialize) {
		if (res->n_out > out_capacity) {
			pg_free_async(ctx, s, tile_counts); pg_free_async(ctx, s, acc);
			return pg_fail(ctx, PG_ERR_OUTPUT_FULL, "pg_hashjoin_probe: output capacity too small");
		}
		k_probe_general<true><<<(unsigned) ntiles, HJ_THREADS, 0, s>>>((const char*) S->data, S->n, S->width,
				S->key_off, S->key_bytes, ht->slots, ht->log2cap, ht->side, ht->nside, pc, ht->inline_val,
				ht->R, ht->wR, tile_counts, (char*) out, acc + 1, -1, ctx->d_status);
		PG_LAUNCHED(ctx);
		if ((rc = pg_check_status(ctx, s, "pg_hashjoin_probe"))) return rc;
	}
	pg_free_async(ctx, s, tile_counts);
	pg_free_async(ctx, s, acc);
	return PG_OK;
}

// pg_hashjoin_probe; a speculative table is settled (and possibly rebuilt)
// when the probe's kernel cannot take it or its checks failed.
static int hj_probe(pg_ctx* ctx, pg_stream stream, pg_hashtable* ht,
		const pg_rel* S, const pg_col* proj, int nproj,
		void* out, uint64_t out_capacity, int flags, int sum_col, pg_join_result* res, const PgPred16* pred)
{
	int rc = hj_probe_run(ctx, stream, ht, S, proj, nproj, out, out_capacity, flags, sum_col, res, pred);
	if (rc != HJ_NEED_SETTLE && rc != HJ_SPEC_REFUTED) return rc;
	if ((rc = hj_settle(ctx, ht))) return rc;
	return hj_probe_run(ctx, stream, ht, S, proj, nproj, out, out_capacity, flags, sum_col, res, pred);
}

extern "C" int pg_hashjoin_probe(pg_ctx* ctx, pg_stream stream, pg_hashtable* ht,
		const pg_rel* S, const pg_col* proj, int nproj,
		void* out, uint64_t out_capacity, int flags, int sum_col, pg_join_result* res)
{
	return hj_probe(ctx, stream, ht, S, proj, nproj, out, out_capacity, flags, sum_col, res, nullptr);
}

extern "C" int pg_hashjoin_probe_where(pg_ctx* ctx, pg_stream stream, pg_hashtable* ht, const pg_rel* S,
		const pg_pred* preds, int npred, const pg_col* proj, int nproj,
		void* out, uint64_t out_capacity, int flags, int sum_col, pg_join_result* res)
{
	if (!ctx || !ht || !S || !res) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_probe_where: null argument");
	if (npred == 0)
		return hj_probe(ctx, stream, ht, S, proj, nproj, out, out_capacity, flags, sum_col, res, nullptr);
	int rc;
	if ((rc = hj_settle(ctx, ht))) return rc;
	PgPredSet P;
	bool has_char = false;
	if ((rc = pg_pred_prepare(ctx, preds, npred, S->width, &P, &has_char))) return rc;
	if ((rc = hj_validate_rel(ctx, S, "pg_hashjoin_probe_where"))) return rc;
	if ((rc = hj_validate_proj(ctx, proj, nproj, ht->wR, S->width))) return rc;
	HjCols pc;
	if ((rc = hj_make_cols(ctx, ht, proj, nproj, &pc))) return rc;
	const bool materialize = (flags & PG_JOIN_MATERIALIZE) != 0;
	PgPred16 p16;
	// In the probe kernel when its register-loading dense path runs: 16-byte
	// tuples and rows, numeric predicates, room for a row per probe tuple.
	const bool fused = ht->unique && ht->inline_val && ht->dense && S->width == 16 &&
		(S->key_off == 0 || S->key_off == 8) && S->key_bytes == 8 && pc.ow_words == 4 &&
		(reinterpret_cast<uintptr_t>(S->data) & 15) == 0 &&
		(!materialize || (out_capacity >= S->n && (reinterpret_cast<uintptr_t>(out) & 15) == 0)) &&
		pg_pred_as16(preds, npred, &p16);
	if (fused)
		return hj_probe(ctx, stream, ht, S, proj, nproj, out, out_capacity, flags, sum_col, res, &p16);
	// Otherwise the filtered probe side first, then the plain probe.
	cudaStream_t s = (cudaStream_t) stream;
	void* tmp = nullptr;
	if ((rc = pg_alloc_async(ctx, s, &tmp, std::max<uint64_t>(S->n, 1) * S->width))) return rc;
	uint64_t m = 0;
	if ((rc = pg_filter(ctx, stream, S, preds, npred, tmp, &m))) { pg_free_async(ctx, s, tmp); return rc; }
	pg_rel F = *S;
	F.data = tmp;
	F.n = m;
	rc = hj_probe(ctx, stream, ht, &F, proj, nproj, out, out_capacity, flags, sum_col, res, nullptr);
	pg_free_async(ctx, s, tmp);
	return rc;
}

// Probe side held as separate arrays (the chunks several threads uploaded):
// one launch per span, all reserving output ranges from one cursor, then one
// readback. Unique-key tables only, where every probe kernel but the
// positional 16-byte one writes through the cursor; with counts == nullptr
// hj_launch_unique never takes the positional path.
extern "C" int pg_hashjoin_probe_spans(pg_ctx* ctx, pg_stream stream, pg_hashtable* ht, const pg_rel* spans,
		int nspans, const pg_col* proj, int nproj, void* out, uint64_t out_capacity, int flags, int sum_col,
		pg_join_result* res)
{
	if (!ctx || !ht || !res || (nspans > 0 && !spans) || nspans < 0)
		return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_probe_spans: null argument");
	if (int rs = hj_settle(ctx, ht)) return rs;
	if (!ht->unique || !ht->inline_val)
		return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_hashjoin_probe_spans: the table has repeated keys");
	res->n_out = 0; res->sum = 0;
	if (nspans == 0) return PG_OK;
	int rc;
	for (int i = 0; i < nspans; ++i) {
		if ((rc = hj_validate_rel(ctx, &spans[i], "pg_hashjoin_probe_spans"))) return rc;
		if (spans[i].width != spans[0].width || spans[i].key_off != spans[0].key_off ||
				spans[i].key_bytes != spans[0].key_bytes)
			return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_probe_spans: spans of different layouts");
	}
	if ((rc = hj_validate_proj(ctx, proj, nproj, ht->wR, spans[0].width))) return rc;
	HjCols pc;
	if ((rc = hj_make_cols(ctx, ht, proj, nproj, &pc))) return rc;
	const bool materialize = (flags & PG_JOIN_MATERIALIZE) != 0;
	if (sum_col >= nproj) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_probe_spans: sum_col out of range");
	if (!(flags & PG_JOIN_SUM)) sum_col = -1;
	if (materialize && out_capacity && !out) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_probe_spans: null output");
	cudaStream_t s = (cudaStream_t) stream;
	unsigned long long* acc = nullptr;   // [cursor, count, sum, spare]
	if ((rc = pg_alloc_async(ctx, s, (void**) &acc, 64))) return rc;
	PG_CUDA(ctx, cudaMemsetAsync(acc, 0, 64, s));
	const bool fold = materialize && (sum_col >= 0 || (flags & PG_JOIN_COUNT));
	for (int pass = 0; pass < (fold ? 2 : 1); ++pass) {
		const bool m = materialize && pass == 0;
		for (int i = 0; i < nspans && !rc; ++i) {
			const pg_rel& S = spans[i];
			if (!S.n) continue;
			rc = hj_launch_unique(ctx, s, ht, (const char*) S.data, S.n, S.width, S.key_off, S.key_bytes, pc,
					m ? (char*) out : nullptr, m ? out_capacity : 0, acc, m, m ? -1 : sum_col);
		}
	}
	unsigned long long h[4] = {0, 0, 0, 0};
	if (!rc) {
		PG_CUDA(ctx, cudaMemcpyAsync(h, acc, 32, cudaMemcpyDeviceToHost, s));
		rc = pg_check_status(ctx, s, "pg_hashjoin_probe_spans");
	}
	pg_free_async(ctx, s, acc);
	if (rc) return rc;
	res->n_out = materialize ? h[0] : h[1];
	res->sum = (int64_t) h[2];
	if (materialize && res->n_out > out_capacity)
		return pg_fail(ctx, PG_ERR_OUTPUT_FULL, "pg_hashjoin_probe_spans: output capacity too small");
	return PG_OK;
}

// ---------------------------------------------------------------------------
// Whole join through host buffers: build from R, then stream S through the
// device in chunks on three streams so that the host->device copy of chunk
// i+1, the probe of chunk i and the device->host copy of chunk i-1 overlap.
// ---------------------------------------------------------------------------
#define HJH_CHUNK (8ull << 20)

extern "C" int pg_hashjoin_host(pg_ctx* ctx, const pg_rel* Rh, const pg_rel* Sh,
		const pg_col* proj, int nproj, void* out_host, uint64_t out_capacity,
		int flags, int sum_col, pg_join_result* res)
{
	if (!ctx || !Rh || !Sh || !res) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_host: null argument");
	int rc;
	if ((rc = hj_validate_proj(ctx, proj, nproj, Rh->width, Sh->width))) return rc;
	const bool materialize = (flags & PG_JOIN_MATERIALIZE) != 0;
	if (materialize && out_capacity && !out_host) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_host: null output");
	uint32_t ow = 0;
	for (int i = 0; i < nproj; ++i) ow += proj[i].bytes;
	res->n_out = 0; res->sum = 0;
	cudaStream_t sin, scomp, sout;
	PG_CUDA(ctx, cudaStreamCreateWithFlags(&sin, cudaStreamNonBlocking));
	PG_CUDA(ctx, cudaStreamCreateWithFlags(&scomp, cudaStreamNonBlocking));
	PG_CUDA(ctx, cudaStreamCreateWithFlags(&sout, cudaStreamNonBlocking));
	char *dR = nullptr, *dS[2] = {nullptr, nullptr}, *dO[2] = {nullptr, nullptr};
	uint64_t* dC[2] = {nullptr, nullptr};     // per-chunk match counts of a positional probe
	bool posit[2] = {false, false};
	unsigned long long* acc = nullptr;        // per chunk slot: [cursor, count, sum, pad] x 2
	unsigned long long* hacc = nullptr;       // pinned copy of acc
	pg_hashtable* ht = nullptr;
	cudaEvent_t ev_in[2], ev_comp[2], ev_out[2];
	for (int i = 0; i < 2; ++i) {
		cudaEventCreateWithFlags(&ev_in[i], cudaEventDisableTiming);
		cudaEventCreateWithFlags(&ev_comp[i], cudaEventDisableTiming);
		cudaEventCreateWithFlags(&ev_out[i], cudaEventDisableTiming);
	}
	auto cleanup = [&]() {
		cudaStreamSynchronize(sin); cudaStreamSynchronize(scomp); cudaStreamSynchronize(sout);
		if (ht) pg_hashtable_free(ctx, ht);
		cudaFree(dR); cudaFree(dS[0]); cudaFree(dS[1]); cudaFree(dO[0]); cudaFree(dO[1]); cudaFree(acc);
		cudaFree(dC[0]); cudaFree(dC[1]);
		if (hacc) cudaFreeHost(hacc);
		for (int i = 0; i < 2; ++i) { cudaEventDestroy(ev_in[i]); cudaEventDestroy(ev_comp[i]); cudaEventDestroy(ev_out[i]); }
		cudaStreamDestroy(sin); cudaStreamDestroy(scomp); cudaStreamDestroy(sout);
	};
#define HJH_TRY(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) { int r_ = pg_cuda_fail(ctx, e_, #call); cleanup(); return r_; } } while (0)
	const uint64_t nR = Rh->n, nS = Sh->n;
	HJH_TRY(cudaMalloc(&dR, std::max<uint64_t>(16, nR * Rh->width)));
	HJH_TRY(cudaMemcpyAsync(dR, Rh->data, nR * Rh->width, cudaMemcpyHostToDevice, scomp));
	pg_rel R = *Rh; R.data = dR;
	if ((rc = pg_hashjoin_build(ctx, scomp, &R, proj, nproj, &ht))) { cleanup(); return rc; }
	if ((rc = hj_settle(ctx, ht))) { cleanup(); return rc; }
	HjCols pc;
	if ((rc = hj_make_cols(ctx, ht, proj, nproj, &pc))) { cleanup(); return rc; }
	if (!(flags & PG_JOIN_SUM)) sum_col = -1;
	const uint64_t CH = std::min<uint64_t>(HJH_CHUNK, std::max<uint64_t>(nS, 1));
	const bool pipelined = ht->unique && ht->inline_val;
	if (!pipelined) {
		// Duplicate keys: sizes are unknown until counted; one device pass.
		char* dSall = nullptr;
		HJH_TRY(cudaMalloc(&dSall, std::max<uint64_t>(16, nS * Sh->width)));
		dS[0] = dSall;
		HJH_TRY(cudaMemcpyAsync(dSall, Sh->data, nS * Sh->width, cudaMemcpyHostToDevice, scomp));
		pg_rel S = *Sh; S.data = dSall;
		char* dOut = nullptr;
		pg_join_result r0;
		if ((rc = pg_hashjoin_probe(ctx, scomp, ht, &S, proj, nproj, nullptr, 0, flags & ~PG_JOIN_MATERIALIZE, sum_col, &r0))) { cleanup(); return rc; }
		if (materialize && r0.n_out) {
			if (r0.n_out > out_capacity) { cleanup(); res->n_out = r0.n_out; return pg_fail(ctx, PG_ERR_OUTPUT_FULL, "pg_hashjoin_host: output capacity too small"); }
			HJH_TRY(cudaMalloc(&dOut, r0.n_out * ow));
			dO[0] = dOut;
			if ((rc = pg_hashjoin_probe(ctx, scomp, ht, &S, proj, nproj, dOut, r0.n_out, PG_JOIN_MATERIALIZE, -1, &r0))) { cleanup(); return rc; }
			HJH_TRY(cudaMemcpyAsync(out_host, dOut, r0.n_out * ow, cudaMemcpyDeviceToHost, scomp));
			HJH_TRY(cudaStreamSynchronize(scomp));
		}
		*res = r0;
		cleanup();
		return PG_OK;
	}
	for (int i = 0; i < 2; ++i) {
		HJH_TRY(cudaMalloc(&dS[i], CH * Sh->width));
		if (materialize) HJH_TRY(cudaMalloc(&dO[i], CH * ow));
		HJH_TRY(cudaMalloc(&dC[i], pg_div_up(CH, PW_CHUNK) * 8));
	}
	HJH_TRY(cudaMalloc(&acc, 2 * 4 * sizeof(unsigned long long)));
	HJH_TRY(cudaMallocHost(&hacc, 2 * 4 * sizeof(unsigned long long)));
	HJH_TRY(cudaStreamSynchronize(scomp));
	const uint64_t nchunks = pg_div_up(nS, CH);
	uint64_t written = 0;
	unsigned long long count = 0, sum = 0;
	auto issue = [&](uint64_t c) -> int {
		const int b = (int) (c & 1);
		const uint64_t r0 = c * CH, rows = std::min<uint64_t>(CH, nS - r0);
		if (c >= 2) HJH_TRY(cudaStreamWaitEvent(sin, ev_comp[b], 0));     // input buffer free
		HJH_TRY(cudaMemcpyAsync(dS[b], (const char*) Sh->data + r0 * Sh->width, rows * Sh->width,
				cudaMemcpyHostToDevice, sin));
		HJH_TRY(cudaEventRecord(ev_in[b], sin));
		HJH_TRY(cudaStreamWaitEvent(scomp, ev_in[b], 0));
		if (c >= 2) HJH_TRY(cudaStreamWaitEvent(scomp, ev_out[b], 0));   // output buffer free
		HJH_TRY(cudaMemsetAsync(acc + 4 * b, 0, 32, scomp));
		if (materialize && hj_launch_unique(ctx, scomp, ht, dS[b], rows, Sh->width, Sh->key_off, Sh->key_bytes,
				pc, dO[b], CH, acc + 4 * b, true, -1, dC[b], &posit[b])) { cleanup(); return PG_ERR_CUDA; }
		if ((!materialize || sum_col >= 0 || (flags & PG_JOIN_COUNT)) &&
				hj_launch_unique(ctx, scomp, ht, dS[b], rows, Sh->width, Sh->key_off, Sh->key_bytes,
				pc, nullptr, 0, acc + 4 * b, false, sum_col)) { cleanup(); return PG_ERR_CUDA; }
		HJH_TRY(cudaGetLastError());
		HJH_TRY(cudaMemcpyAsync(hacc + 4 * b, acc + 4 * b, 32, cudaMemcpyDeviceToHost, scomp));
		HJH_TRY(cudaEventRecord(ev_comp[b], scomp));
		return PG_OK;
	};
	if (nchunks && (rc = issue(0))) return rc;
	for (uint64_t c = 0; c < nchunks; ++c) {
		const int b = (int) (c & 1);
		if (c + 1 < nchunks && (rc = issue(c + 1))) return rc;
		HJH_TRY(cudaEventSynchronize(ev_comp[b]));
		const unsigned long long rows_out = hacc[4 * b];
		count += materialize ? rows_out : hacc[4 * b + 1];
		if (!materialize || sum_col >= 0 || (flags & PG_JOIN_COUNT)) sum += hacc[4 * b + 2];
		if (materialize && rows_out) {
			if (written + rows_out > out_capacity) { written += rows_out; continue; }
			const uint64_t rows_in = std::min<uint64_t>(CH, nS - c * CH);
			if (posit[b] && rows_out < rows_in) {
				// Some probe tuples missed: close the gaps before copying out.
				if ((rc = hj_compact(ctx, scomp, dO[b], rows_in, dC[b], rows_out))) { cleanup(); return rc; }
				HJH_TRY(cudaEventRecord(ev_comp[b], scomp));
			}
			HJH_TRY(cudaStreamWaitEvent(sout, ev_comp[b], 0));
			HJH_TRY(cudaMemcpyAsync((char*) out_host + written * ow, dO[b], rows_out * ow, cudaMemcpyDeviceToHost, sout));
			written += rows_out;
		}
		HJH_TRY(cudaEventRecord(ev_out[b], sout));
	}
	HJH_TRY(cudaStreamSynchronize(sout));
	if ((rc = pg_check_status(ctx, scomp, "pg_hashjoin_host"))) { cleanup(); return rc; }
	if (materialize && (flags & PG_JOIN_COUNT) == 0 && sum_col < 0) count = written;
	res->n_out = materialize ? written : count;
	res->sum = (int64_t) sum;
	cleanup();
#undef HJH_TRY
	if (materialize && written > out_capacity)
		return pg_fail(ctx, PG_ERR_OUTPUT_FULL, "pg_hashjoin_host: output capacity too small");
	return PG_OK;
}

// ---------------------------------------------------------------------------
// Join then group-by in one pass (a HashJoinOp feeding AggregateSum /
// AggregateCount: join.cpp:503-562 with genericaggregate.cpp:240-282). The
// group key is the table's value (the one projected build column); a narrow
// dense table stores value - vmin, which is the row's group slot directly. The
// probe-side value is folded into a dense group table with the atomics of the
// group-by (a dec value as an exact count of units 2^s in four words: for a
// value near the column's largest, one returning atomic), so the join rows
// are never written.
// ---------------------------------------------------------------------------
template <int VT, int AGG>
__global__ void __launch_bounds__(PW_WARPS * 32, 4)
k_probe16_groupby(const char* __restrict__ S, uint64_t n, uint32_t koff, const HjProbeTable tb, uint32_t voff,
		uint32_t goff, unsigned long long* __restrict__ acc, uint64_t wst, PgFx fx, unsigned char* __restrict__ present)
{
	constexpr bool DEC = AGG == PG_AGG_SUM && VT == PG_VAL_DEC;
	constexpr int ITEMS = PW_CHUNK / 32;
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint64_t nchunks = pg_div_up(n, PW_CHUNK);
	const uint64_t W = (uint64_t) gridDim.x * PW_WARPS;
	const uint64_t first = (uint64_t) blockIdx.x * PW_WARPS + warp;
	const uint64_t keep = pg_policy_evict_last();
	const uint64_t instream = pg_policy_evict_first();
	if (first >= nchunks) return;
	const int fs = DEC ? fx.p[0] : 0, fb = DEC ? fx.p[1] : 0;
	uint32_t fl = 0;
	uint4 cur[ITEMS], nxt[ITEMS];
	auto load = [&](uint64_t c, uint4 (&t)[ITEMS]) {
		const uint32_t rows = (uint32_t) pg_min64(PW_CHUNK, n - c * PW_CHUNK);
		#pragma unroll
		for (int j = 0; j < ITEMS; ++j) {
			const uint32_t p = j * 32 + lane;
			t[j] = p < rows ? hj_ld_stream(S + (c * PW_CHUNK + p) * 16, instream) : make_uint4(0, 0, 0, 0);
		}
	};
	load(first, cur);
	for (uint64_t c = first; c < nchunks; c += W) {
		if (c + W < nchunks) load(c + W, nxt);
		const uint32_t rows = (uint32_t) pg_min64(PW_CHUNK, n - c * PW_CHUNK);
		uint32_t e[ITEMS];
		#pragma unroll
		for (int j = 0; j < ITEMS; ++j) {
			const uint4 t = cur[j];
			const int64_t key = koff == 0 ? (int64_t) (((uint64_t) t.y << 32) | t.x) : (int64_t) (((uint64_t) t.w << 32) | t.z);
			const unsigned long long d = (unsigned long long) key - (unsigned long long) tb.dmin;
			e[j] = 0xFFFFFFFFu;
			if (j * 32 + lane < rows && d < tb.drange)
				asm("ld.global.nc.L1::no_allocate.L2::cache_hint.u32 %0, [%1], %2;"
						: "=r"(e[j]) : "l"(tb.dense32 + d), "l"(keep));
			if (e[j] != 0xFFFFFFFFu) e[j] -= goff;      // group slot: value - smallest value
		}
		if (DEC) {
			// PG_FX_WORDS words per group, word k at acc[group + k * wst]
			// (pg_fx_atomic_add_rows): a value near the column's largest is one
			// returning add; the first add into a group returns the initial 0
			// and marks it present once.
			pg_fx3 f[ITEMS];
			uint64_t slot[ITEMS];
			bool ok[ITEMS];
			#pragma unroll
			for (int j = 0; j < ITEMS; ++j) {
				const uint4 t = cur[j];
				ok[j] = e[j] != 0xFFFFFFFFu;
				slot[j] = ok[j] ? e[j] : 0;
				f[j] = ok[j] ? pg_fx_take(voff == 0 ? (((uint64_t) t.y << 32) | t.x) : (((uint64_t) t.w << 32) | t.z),
				                          fs, fb, fl)
				             : pg_fx3{0, 0, 0};
			}
			pg_fx_atomic_add_rows<ITEMS>(acc, wst, slot, 1, ok, f, present);
		} else {
			#pragma unroll
			for (int j = 0; j < ITEMS; ++j) {
				if (e[j] == 0xFFFFFFFFu) continue;
				const uint4 t = cur[j];
				if (AGG == PG_AGG_COUNT) { atomicAdd(&acc[e[j]], 1ull); continue; }
				const uint32_t w = voff / 4;
				const uint32_t w0 = w == 0 ? t.x : w == 1 ? t.y : w == 2 ? t.z : t.w;
				if (VT == PG_VAL_INT) atomicAdd(reinterpret_cast<unsigned int*>(&acc[e[j]]), w0);
				else atomicAdd(&acc[e[j]], ((unsigned long long) (w == 0 ? t.y : t.w) << 32) | w0);
				present[e[j]] = 1;
			}
		}
		#pragma unroll
		for (int j = 0; j < ITEMS; ++j) cur[j] = nxt[j];
	}
	if (fl) atomicOr(reinterpret_cast<unsigned int*>(fx.p + 2), fl);
}

extern "C" int pg_hashjoin_groupby(pg_ctx* ctx, pg_stream stream, pg_hashtable* ht, const pg_rel* S,
		uint32_t val_off, int val_type, int agg, void* out, uint64_t out_capacity, uint64_t* ngroups)
{
	if (!ctx || !ht || !S || !ngroups) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_groupby: null argument");
	int rc;
	if ((rc = hj_validate_rel(ctx, S, "pg_hashjoin_groupby"))) return rc;
	if (agg != PG_AGG_SUM && agg != PG_AGG_COUNT) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_groupby: bad aggregate");
	if (agg == PG_AGG_SUM && (val_type < 0 || val_type > 2 || (val_type == PG_VAL_INT ? (val_off & 3) : (val_off & 7)) ||
			val_off + (val_type == PG_VAL_INT ? 4 : 8) > S->width))
		return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_groupby: bad value column");
	*ngroups = 0;
	if ((rc = hj_settle(ctx, ht))) return rc;
	const uint64_t vrange = ht->dense32 ? ht->vmax - ht->vlo + 1 : 0;
	uint32_t gbytes = 0;
	for (int c = 0; c < ht->bcols.n; ++c) gbytes += 4 * ht->bcols.words[c];
	if (!ht->dense32 || ht->bcols.n != 1 || (gbytes != 4 && gbytes != 8) || vrange == 0 ||
			vrange > std::max<uint64_t>(4 * ht->nbuild, 1 << 20) || vrange > (1ull << 28) ||
			S->width != 16 || (S->key_off != 0 && S->key_off != 8) || S->key_bytes != 8 ||
			(reinterpret_cast<uintptr_t>(S->data) & 15) != 0)
		return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_hashjoin_groupby: needs a narrow dense table with one build "
				"column of compact range and 16-byte probe tuples");
	cudaStream_t s = (cudaStream_t) stream;
	const bool dec = agg == PG_AGG_SUM && val_type == PG_VAL_DEC;
	char* mem = nullptr;
	const uint64_t words = vrange * (dec ? PG_FX_WORDS : 1);
	const size_t pres_end = (words + 1) * 8 + ((vrange + 15) & ~15ull);
	const size_t bytes = pres_end + 16;
	if ((rc = pg_alloc_async(ctx, s, (void**) &mem, bytes))) return rc;
	unsigned long long* acc = reinterpret_cast<unsigned long long*>(mem);   // a dec sum: word k of group g at acc[g + k vrange]
	unsigned long long* cursor = acc + words;
	unsigned char* present = reinterpret_cast<unsigned char*>(cursor + 1);
	PgFx fx = {reinterpret_cast<int*>(mem + pres_end)};
	// A dec sum's unit: the probe column's largest exponent, from every 1024th
	// tuple (4x margin) on large inputs; redone exactly if a value lies above.
	const bool sampled = S->n >= (1ull << 22);
	for (int pass = 0; pass < 2; ++pass) {
		PG_CUDA(ctx, cudaMemsetAsync(mem, 0, pres_end, s));
		if (dec && (rc = pg_fx_prepare(ctx, s, (const char*) S->data, S->n, 16, val_off, pass == 0 && sampled ? 1024 : 1,
				2, fx))) return rc;
		if (S->n) {
			HjProbeTable tb = {};
			tb.dense32 = ht->dense32; tb.vmin = ht->vmin; tb.dmin = ht->dmin; tb.drange = ht->drange;
			const int grid = (int) std::min<uint64_t>(pg_div_up(pg_div_up(S->n, PW_CHUNK), PW_WARPS), (uint64_t) ctx->sm_count * 24);
#define PG_LAUNCH(VT, AGG) k_probe16_groupby<VT, AGG><<<grid, PW_WARPS * 32, 0, s>>>((const char*) S->data, S->n, \
					S->key_off, tb, val_off, (uint32_t) (ht->vlo - ht->vmin), acc, vrange, fx, present)
			if (agg == PG_AGG_COUNT) PG_LAUNCH(PG_VAL_LONG, PG_AGG_COUNT);
			else if (val_type == PG_VAL_INT) PG_LAUNCH(PG_VAL_INT, PG_AGG_SUM);
			else if (val_type == PG_VAL_LONG) PG_LAUNCH(PG_VAL_LONG, PG_AGG_SUM);
			else PG_LAUNCH(PG_VAL_DEC, PG_AGG_SUM);
#undef PG_LAUNCH
			PG_LAUNCHED(ctx);
		}
		if ((rc = pg_dense_groups_emit(ctx, s, acc, fx, present, vrange, (long long) ht->vlo, gbytes, val_type, agg,
				out, out_capacity, cursor))) return rc;
		unsigned long long ng = 0;
		unsigned int fl = 0;
		PG_CUDA(ctx, cudaMemcpyAsync(&ng, cursor, 8, cudaMemcpyDeviceToHost, s));
		if (dec) PG_CUDA(ctx, cudaMemcpyAsync(&fl, fx.p + 2, 4, cudaMemcpyDeviceToHost, s));
		if ((rc = pg_check_status(ctx, s, "pg_hashjoin_groupby"))) return rc;
		*ngroups = ng;
		if ((fl & PG_FX_RANGE) && pass == 0) continue;
		pg_free_async(ctx, s, mem);
		if (fl & PG_FX_SPECIALS)
			return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_hashjoin_groupby: infinities or NaNs in the summed column "
					"(probe, then pg_groupby)");
		if (ng > out_capacity) return pg_fail(ctx, PG_ERR_OUTPUT_FULL, "pg_hashjoin_groupby: output capacity too small");
		return PG_OK;
	}
	pg_free_async(ctx, s, mem);
	return pg_fail(ctx, PG_ERR_CUDA, "pg_hashjoin_groupby: dec sum unit refuted twice");
}
