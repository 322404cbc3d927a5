// MPSM / sort-merge join on sm_103a.
//
// Replaces SortMergeJoinOp::BufferAndSort (operators/join.cpp:945-996) and
// the merge loops of OldMPSMJoinOp / MPSMJoinOp (join.cpp:1245-1371,
// 1516-1538; PresortedPrepartitionedMergeJoinOp::getNext, join.cpp:1929-1968),
// which sort per-thread runs of both inputs and merge each build run against
// the probe runs, buffering the build tuples of the current key
// (mostfreqbuildkeyoccurances) and emitting the cartesian product of equal-key
// groups.
//
// Count/sum joins whose key span is 2^13..2^24 values take the bucketed form
// further down (high-bit sort + shared-memory merge of 4096-key buckets).
//
// GPU plan: sort both relations (pg_sort.cu), cut each sorted relation into
// equal-key runs (stream compaction of run heads: run starts and run keys),
// match build runs to probe runs by merging the two sorted run-key arrays, scan the per-run output counts |R_k|*|S_k|, and either fold
// count and sum (no output materialised; a build column sums as
// |S_k| * sum_R_k, a probe column as |R_k| * sum_S_k, wrapping int64 like the
// reference's CtLong +=) or write every pair, each thread producing a
// contiguous slice of output positions (load-balanced over skewed groups).
// The reference's per-key buffer limit does not exist here: any multiplicity
// is joined.
#include "pg_internal.cuh"
#include "pg_sort.cuh"
#include <algorithm>

#define MJ_MAX_COLS 16

struct MjCols {
	int n, ow_words;
	uint8_t side[MJ_MAX_COLS];
	uint16_t off[MJ_MAX_COLS];    // byte offset in the side's tuple
	uint8_t words[MJ_MAX_COLS];
};

struct MjSide {
	const pg_rec* rec;   // sorted records
	const char* rows;    // original tuples
	uint32_t W, koff;
	int mode;            // pg_sort_mode
	const uint64_t* run_start;  // [nruns + 1]
	uint64_t nruns;
};

// Word w of column (off, words) of the tuple behind record r.
__device__ __forceinline__ uint32_t mj_word(const MjSide& sd, const pg_rec& r, uint32_t off, uint32_t w)
{
	if (sd.mode == 2) return reinterpret_cast<const uint32_t*>(sd.rows + r.val * sd.W + off)[w];
	// 16-byte tuple: the key half and the other half.
	uint32_t byte = off + 4 * w;
	bool in_key = (byte >= sd.koff && byte < sd.koff + 8);
	unsigned long long half = in_key ? (unsigned long long) r.key : r.val;
	uint32_t rel = in_key ? byte - sd.koff : (byte >= 8 ? byte - 8 : byte);
	return rel == 0 ? (uint32_t) half : (uint32_t) (half >> 32);
}

__device__ __forceinline__ unsigned long long mj_col64(const MjSide& sd, const pg_rec& r, uint32_t off, uint32_t words)
{
	uint32_t lo = mj_word(sd, r, off, 0);
	if (words == 2) return ((unsigned long long) mj_word(sd, r, off, 1) << 32) | lo;
	return (unsigned long long) (long long) (int32_t) lo;
}

// Equal-key runs of a sorted record array by stream compaction over chunks of
// MJ_RUN_CHUNK records: k_run_count counts run heads per chunk, a scan of the
// chunk counts gives each chunk its first run id, and k_run_write writes, in
// order, every run's first record index and key.
#define MJ_RUN_CHUNK 4096
#define MJ_RUN_THREADS 256

__device__ __forceinline__ bool mj_head(const pg_rec* rec, uint64_t i)
{
	return i == 0 || rec[i].key != rec[i - 1].key;
}

__global__ void __launch_bounds__(MJ_RUN_THREADS)
k_run_count(const pg_rec* __restrict__ rec, uint64_t n, uint64_t* __restrict__ ccount)
{
	__shared__ uint32_t wsum[MJ_RUN_THREADS / 32];
	const uint64_t nchunks = pg_div_up(n, MJ_RUN_CHUNK);
	for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
		const uint64_t lo = c * MJ_RUN_CHUNK, hi = pg_min64(n, lo + MJ_RUN_CHUNK);
		uint32_t cnt = 0;
		for (uint64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) cnt += mj_head(rec, i);
		#pragma unroll
		for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
		if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = cnt;
		__syncthreads();
		if (threadIdx.x == 0) {
			uint64_t t = 0;
			for (int w = 0; w < MJ_RUN_THREADS / 32; ++w) t += wsum[w];
			ccount[c] = t;
		}
		__syncthreads();
	}
}

__global__ void __launch_bounds__(MJ_RUN_THREADS)
k_run_write(const pg_rec* __restrict__ rec, uint64_t n, const uint64_t* __restrict__ cfirst,
		uint64_t* __restrict__ start, long long* __restrict__ rkey)
{
	__shared__ uint32_t wsum[MJ_RUN_THREADS / 32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint64_t nchunks = pg_div_up(n, MJ_RUN_CHUNK);
	for (uint64_t c = blockIdx.x; c < nchunks; c += gridDim.x) {
		const uint64_t lo = c * MJ_RUN_CHUNK, hi = pg_min64(n, lo + MJ_RUN_CHUNK);
		uint64_t base = cfirst[c];
		for (uint64_t i0 = lo; i0 < hi; i0 += blockDim.x) {
			const uint64_t i = i0 + threadIdx.x;
			const bool h = i < hi && mj_head(rec, i);
			const uint32_t ball = __ballot_sync(0xffffffffu, h);
			if (lane == 0) wsum[warp] = __popc(ball);
			__syncthreads();
			uint32_t before = 0, total = 0;
			#pragma unroll
			for (int w = 0; w < MJ_RUN_THREADS / 32; ++w) { const uint32_t x = wsum[w]; before += w < warp ? x : 0; total += x; }
			if (h) {
				const uint64_t id = base + before + __popc(ball & ((1u << lane) - 1));
				start[id] = i;
				rkey[id] = rec[i].key;
			}
			base += total;
			__syncthreads();
		}
	}
}

// For every build run: matching probe run (or none), output count, and the
// folded count/sum contribution. A warp takes MJ_WARP_RUNS consecutive build
// runs: one lane finds the window of probe runs whose keys lie in the batch's
// key range (two binary searches), then the lanes take consecutive build runs
// (coalesced reads of keys and starts, coalesced count/match writes) and
// binary-search their key inside the window, which stays in L1. The summed
// column of a matched run is added by its lane when the run is short, and by
// the whole warp (strided loads, shuffle reduction) when it is long, so skewed
// keys do not serialise on one lane.
#define MJ_WARP_RUNS 512
#define MJ_SHORT_RUN 64

__device__ __forceinline__ uint64_t mj_lower(const long long* __restrict__ K, uint64_t lo, uint64_t hi, long long k)
{
	while (lo < hi) {
		const uint64_t mid = (lo + hi) >> 1;
		if (K[mid] < k) lo = mid + 1; else hi = mid;
	}
	return lo;
}

__global__ void __launch_bounds__(256)
k_match_runs(MjSide R, MjSide S, const long long* __restrict__ RK, const long long* __restrict__ SK,
		MjCols pc, int sum_col, uint64_t* __restrict__ counts, uint64_t* __restrict__ match,
		unsigned long long* __restrict__ agg)
{
	const int lane = threadIdx.x & 31;
	const uint64_t gwarp = ((uint64_t) blockIdx.x * blockDim.x + threadIdx.x) >> 5;
	const uint64_t nwarps = ((uint64_t) gridDim.x * blockDim.x) >> 5;
	const bool sum_r = sum_col >= 0 && pc.side[sum_col] == 0, sum_s = sum_col >= 0 && pc.side[sum_col] != 0;
	const uint32_t soff = sum_col >= 0 ? pc.off[sum_col] : 0, swords = sum_col >= 0 ? pc.words[sum_col] : 0;
	unsigned long long sum_acc = 0;
	for (uint64_t u0 = gwarp * MJ_WARP_RUNS; u0 < R.nruns; u0 += nwarps * MJ_WARP_RUNS) {
		const uint64_t u1 = pg_min64(R.nruns, u0 + MJ_WARP_RUNS);
		uint64_t slo = 0, shi = 0;
		if (lane == 0) {
			slo = mj_lower(SK, 0, S.nruns, RK[u0]);
			const long long klast = RK[u1 - 1];
			shi = klast == LLONG_MAX ? S.nruns : mj_lower(SK, slo, S.nruns, klast + 1);
		}
		slo = __shfl_sync(0xffffffffu, slo, 0);
		shi = __shfl_sync(0xffffffffu, shi, 0);
		for (uint64_t j = u0; j < u1; j += 32) {
			const uint64_t u = j + lane;
			const bool valid = u < u1;
			uint64_t c = 0, m = UINT64_MAX, lo_i = 0, hi_i = 0, other = 0;
			if (valid) {
				const long long k = RK[u];
				const uint64_t v = mj_lower(SK, slo, shi, k);
				if (v < shi && SK[v] == k) {
					const uint64_t r0 = R.run_start[u], r1 = R.run_start[u + 1];
					const uint64_t s0 = S.run_start[v], s1 = S.run_start[v + 1];
					c = (r1 - r0) * (s1 - s0);
					m = v;
					if (sum_r) { lo_i = r0; hi_i = r1; other = s1 - s0; }
					else if (sum_s) { lo_i = s0; hi_i = s1; other = r1 - r0; }
				}
				counts[u] = c;
				match[u] = m;
			}
			if (sum_col < 0) continue;
			const MjSide& sd = sum_r ? R : S;
			const bool longrun = hi_i - lo_i > MJ_SHORT_RUN;
			if (!longrun && hi_i > lo_i) {
				unsigned long long part = 0;
				for (uint64_t i = lo_i; i < hi_i; ++i) part += mj_col64(sd, sd.rec[i], soff, swords);
				sum_acc += part * (unsigned long long) other;
			}
			uint32_t longs = __ballot_sync(0xffffffffu, longrun);
			while (longs) {
				const int l = __ffs(longs) - 1;
				longs &= longs - 1;
				const uint64_t a = __shfl_sync(0xffffffffu, lo_i, l), b = __shfl_sync(0xffffffffu, hi_i, l);
				const uint64_t o = __shfl_sync(0xffffffffu, other, l);
				unsigned long long part = 0;
				for (uint64_t i = a + lane; i < b; i += 32) part += mj_col64(sd, sd.rec[i], soff, swords);
				#pragma unroll
				for (int q = 16; q > 0; q >>= 1) part += __shfl_xor_sync(0xffffffffu, part, q);
				if (lane == 0) sum_acc += part * (unsigned long long) o;
			}
		}
	}
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) sum_acc += __shfl_down_sync(0xffffffffu, sum_acc, o);
	if (lane == 0 && sum_acc) atomicAdd(agg, sum_acc);
}

#define MJ_PER_THREAD 8

// Writes output rows [t*8, t*8+8): pair (u, v) of position p is found by a
// binary search over the scanned counts; within a pair, position q maps to
// probe tuple q / |R_u| and build tuple q % |R_u|.
__global__ void k_mj_write(MjSide R, MjSide S, MjCols pc, const uint64_t* __restrict__ offs,
		const uint64_t* __restrict__ match, uint64_t nout, char* __restrict__ out)
{
	const uint64_t ow = (uint64_t) pc.ow_words * 4;
	for (uint64_t t = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; t * MJ_PER_THREAD < nout;
			t += (uint64_t) gridDim.x * blockDim.x) {
		uint64_t p = t * MJ_PER_THREAD;
		const uint64_t pend = pg_min64(nout, p + MJ_PER_THREAD);
		// upper_bound(offs, p) - 1 over runs with offsets
		uint64_t lo = 0, hi = R.nruns;
		while (lo < hi) {
			uint64_t mid = (lo + hi) >> 1;
			if (offs[mid] <= p) lo = mid + 1; else hi = mid;
		}
		uint64_t u = lo - 1;
		while (p < pend) {
			while (offs[u + 1] <= p) ++u;           // skip empty runs
			const uint64_t v = match[u];
			const uint64_t r0 = R.run_start[u], nr = R.run_start[u + 1] - r0;
			const uint64_t s0 = S.run_start[v];
			uint64_t q = p - offs[u];
			const uint64_t stop = pg_min64(pend, offs[u + 1]);
			for (; p < stop; ++p, ++q) {
				const pg_rec& br = R.rec[r0 + q % nr];
				const pg_rec& pr = S.rec[s0 + q / nr];
				uint32_t* o = reinterpret_cast<uint32_t*>(out + p * ow);
				int wo = 0;
				for (int c = 0; c < pc.n; ++c)
					for (int w = 0; w < pc.words[c]; ++w)
						o[wo++] = pc.side[c] ? mj_word(S, pr, pc.off[c], w) : mj_word(R, br, pc.off[c], w);
			}
		}
	}
}

static int mj_runs(pg_ctx* ctx, cudaStream_t s, const pg_rec* rec, uint64_t n, uint64_t** starts,
		long long** keys, uint64_t* nruns)
{
	int rc;
	const uint64_t nchunks = pg_div_up(std::max<uint64_t>(n, 1), MJ_RUN_CHUNK);
	uint64_t* cc = nullptr;
	uint64_t* total = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &cc, (nchunks + 1) * 8))) return rc;
	if ((rc = pg_alloc_async(ctx, s, (void**) &total, 8))) return rc;
	const int blocks = (int) std::min<uint64_t>(nchunks, (uint64_t) ctx->sm_count * 8);
	if (n) { k_run_count<<<blocks, MJ_RUN_THREADS, 0, s>>>(rec, n, cc); PG_LAUNCHED(ctx); }
	else PG_CUDA(ctx, cudaMemsetAsync(cc, 0, 8, s));
	if ((rc = pg_scan_u64(ctx, s, cc, nchunks, total))) return rc;
	uint64_t nr = 0;
	PG_CUDA(ctx, cudaMemcpyAsync(&nr, total, 8, cudaMemcpyDeviceToHost, s));
	PG_CUDA(ctx, cudaStreamSynchronize(s));
	uint64_t* st = nullptr;
	long long* rk = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &st, (nr + 1) * 8))) return rc;
	if ((rc = pg_alloc_async(ctx, s, (void**) &rk, (nr + 1) * 8))) return rc;
	if (n) { k_run_write<<<blocks, MJ_RUN_THREADS, 0, s>>>(rec, n, cc, st, rk); PG_LAUNCHED(ctx); }
	PG_CUDA(ctx, cudaMemcpyAsync(st + nr, &n, 8, cudaMemcpyHostToDevice, s));
	pg_free_async(ctx, s, cc);
	pg_free_async(ctx, s, total);
	*starts = st; *keys = rk; *nruns = nr;
	return PG_OK;
}

// ---------------------------------------------------------------------------
// Count/sum without materialising, for key spans of 2^13 .. 2^24 values: both
// relations are sorted on the bits of (key - kmin) above the low 12 (one
// stable radix partition each, 2..4096 buckets), and each bucket pair, 4096
// consecutive key values, is merged in shared memory: per key, the tuples on
// each side and the summed column; then sum over keys of |R_k| * |S_k| and
// sum_R_k * |S_k| (or sum_S_k * |R_k|). This is the sort-merge of the
// general path with its last radix digit, run detection and run matching
// fused into one pass over both relations.
// ---------------------------------------------------------------------------
#define MJ_LOCAL_BITS 12
#define MJ_LOCAL (1u << MJ_LOCAL_BITS)

__device__ __forceinline__ unsigned long long mj_tuple_col(const char* t, uint32_t off, uint32_t words)
{
	const uint32_t* w = reinterpret_cast<const uint32_t*>(t + off);
	if (words == 2) return ((unsigned long long) w[1] << 32) | w[0];
	return (unsigned long long) (long long) (int32_t) w[0];
}

__global__ void __launch_bounds__(256)
k_mj_bucket_join(const char* __restrict__ R, const uint64_t* __restrict__ roffs, uint32_t wR, uint32_t rkoff,
		uint32_t rkb, const char* __restrict__ S, const uint64_t* __restrict__ soffs, uint32_t wS, uint32_t skoff,
		uint32_t skb, long long kmin, int sum_side, uint32_t soff, uint32_t swords,
		unsigned long long* __restrict__ agg, uint64_t* __restrict__ bucket_rows)
{
	__shared__ unsigned long long btot;
	extern __shared__ __align__(16) unsigned char mj_smem[];
	unsigned long long* sm = reinterpret_cast<unsigned long long*>(mj_smem);    // [MJ_LOCAL]
	uint32_t* cR = reinterpret_cast<uint32_t*>(sm + MJ_LOCAL);                   // [MJ_LOCAL]
	uint32_t* cS = cR + MJ_LOCAL;                                                // [MJ_LOCAL]
	const uint32_t b = blockIdx.x;
	for (uint32_t k = threadIdx.x; k < MJ_LOCAL; k += blockDim.x) { sm[k] = 0; cR[k] = 0; cS[k] = 0; }
	if (threadIdx.x == 0) btot = 0;
	__syncthreads();
	const uint64_t r0 = roffs[b], r1 = roffs[b + 1], s0 = soffs[b], s1 = soffs[b + 1];
	// Eight tuples per thread are loaded before their shared-memory updates,
	// so eight loads are in flight per thread.
	for (int side = 0; side < 2; ++side) {
		const char* base = side ? S : R;
		const uint64_t lo = side ? s0 : r0, hi = side ? s1 : r1;
		const uint32_t w = side ? wS : wR, koff = side ? skoff : rkoff, kb = side ? skb : rkb;
		uint32_t* cnt = side ? cS : cR;
		const bool sums = sum_side == side;
		for (uint64_t i0 = lo + threadIdx.x; i0 < hi; i0 += 8 * (uint64_t) blockDim.x) {
			uint32_t k[8];
			unsigned long long v[8];
			#pragma unroll
			for (int u = 0; u < 8; ++u) {
				const uint64_t i = i0 + (uint64_t) u * blockDim.x;
				k[u] = MJ_LOCAL;
				v[u] = 0;
				if (i < hi) {
					const char* t = base + i * w;
					k[u] = (uint32_t) ((unsigned long long) (pg_load_key(t + koff, kb) - kmin) & (MJ_LOCAL - 1));
					if (sums) v[u] = mj_tuple_col(t, soff, swords);
				}
			}
			#pragma unroll
			for (int u = 0; u < 8; ++u) {
				if (k[u] == MJ_LOCAL) continue;
				atomicAdd(&cnt[k[u]], 1u);
				if (sums) atomicAdd(&sm[k[u]], v[u]);
			}
		}
	}
	__syncthreads();
	unsigned long long c = 0, sum = 0;
	for (uint32_t k = threadIdx.x; k < MJ_LOCAL; k += blockDim.x) {
		const unsigned long long a = cR[k], d = cS[k];
		c += a * d;
		if (sum_side == 0) sum += sm[k] * d;
		else if (sum_side == 1) sum += sm[k] * a;
	}
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		c += __shfl_down_sync(0xffffffffu, c, o);
		sum += __shfl_down_sync(0xffffffffu, sum, o);
	}
	if ((threadIdx.x & 31) == 0) {
		if (c) { atomicAdd(&agg[0], c); atomicAdd(&btot, c); }
		if (sum) atomicAdd(&agg[1], sum);
	}
	if (bucket_rows) {
		__syncthreads();
		if (threadIdx.x == 0) bucket_rows[b] = btot;
	}
}

// offs[b] = first index of the sorted relation whose bucket (key - kmin) >>
// MJ_LOCAL_BITS is >= b, for b in [0, B]; the relation is sorted on the bucket.
__global__ void k_mj_bounds(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t koff, uint32_t kbytes,
		long long kmin, uint32_t B, uint64_t* __restrict__ offs)
{
	const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
	if (b > B) return;
	uint64_t lo = 0, hi = n;
	while (lo < hi) {
		const uint64_t mid = (lo + hi) >> 1;
		const unsigned long long d = (unsigned long long) (pg_load_key(in + mid * W + koff, kbytes) - kmin);
		if ((d >> MJ_LOCAL_BITS) < b) lo = mid + 1; else hi = mid;
	}
	offs[b] = lo;
}

// Key range into mm[0..1] (keys ^ 2^63 as unsigned); with `unsorted`, also
// whether some key is greater than the next one.
__global__ void k_mj_minmax(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t koff, uint32_t kbytes,
		unsigned long long* __restrict__ mm, unsigned long long* __restrict__ unsorted)
{
	unsigned long long lo = ~0ull, hi = 0;
	bool down = false;
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n; i += (uint64_t) gridDim.x * blockDim.x) {
		const long long k = pg_load_key(in + i * W + koff, kbytes);
		const unsigned long long u = (unsigned long long) k ^ (1ull << 63);
		lo = u < lo ? u : lo;
		hi = u > hi ? u : hi;
		if (unsorted && i + 1 < n && k > pg_load_key(in + (i + 1) * W + koff, kbytes)) down = true;
	}
	if (unsorted && __any_sync(0xffffffffu, down) && (threadIdx.x & 31) == 0) *unsorted = 1;
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		const unsigned long long a = __shfl_down_sync(0xffffffffu, lo, o), b = __shfl_down_sync(0xffffffffu, hi, o);
		lo = a < lo ? a : lo;
		hi = b > hi ? b : hi;
	}
	if ((threadIdx.x & 31) == 0) { atomicMin(&mm[0], lo); atomicMax(&mm[1], hi); }
}

// ---------------------------------------------------------------------------
// Materialised MPSM over key buckets (16-byte tuples, 8-byte keys, 16-byte
// output rows). After the bucket partition of both sides (as for the
// count/sum), k_mj_bucket_join writes each bucket's output row count, a scan
// turns them into output offsets, and k_mj_bucket_write joins each bucket
// pair in one CTA: the build side's packed values counting-sorted by key into
// shared memory (a run per key), then every probe tuple writes one row per
// build tuple of its key at a block-scanned position. Output rows are in
// bucket order; within a bucket their order is unspecified (as for every
// join output).
// ---------------------------------------------------------------------------
#define MJW_THREADS 1024
#define MJW_CAP 24576            // build tuples of one bucket held in shared memory (192 KB)

// The build-projected words of a row that are not the join key, packed.
struct MjPack {
	int n;
	uint8_t roff[2];             // word offsets in the build tuple
};

__device__ __forceinline__ uint32_t mjw_word(const uint4& t, uint32_t i)
{
	return i == 0 ? t.x : i == 1 ? t.y : i == 2 ? t.z : t.w;
}

// Output word source: 0-3 probe tuple word, 4-5 packed build word.
__device__ __forceinline__ uint32_t mjw_pick(const uint4& t, unsigned long long v, uint32_t sel)
{
	return sel < 4 ? mjw_word(t, sel) : sel == 4 ? (uint32_t) v : (uint32_t) (v >> 32);
}

// Exclusive scan of x over the CTA's MJW_THREADS threads; *total = the sum.
// wsum: MJW_THREADS / 32 words of shared memory. Ends with a barrier.
__device__ __forceinline__ uint32_t mjw_block_scan(uint32_t x, uint32_t* wsum, uint32_t* total)
{
	const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	uint32_t inc = x;
	#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
		if (lane >= (uint32_t) o) inc += y;
	}
	if (lane == 31) wsum[warp] = inc;
	__syncthreads();
	if (warp == 0) {
		uint32_t w = lane < MJW_THREADS / 32 ? wsum[lane] : 0;
		#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
			if (lane >= (uint32_t) o) w += y;
		}
		if (lane < MJW_THREADS / 32) wsum[lane] = w;
	}
	__syncthreads();
	const uint32_t before = (warp ? wsum[warp - 1] : 0) + inc - x;
	*total = wsum[MJW_THREADS / 32 - 1];
	__syncthreads();
	return before;
}

__global__ void __launch_bounds__(MJW_THREADS, 1)
k_mj_bucket_write(const uint4* __restrict__ R, const uint64_t* __restrict__ roffs, uint32_t rkw, MjPack bp,
		const uint4* __restrict__ S, const uint64_t* __restrict__ soffs, uint32_t skw, long long kmin,
		const uint64_t* __restrict__ bucket_off, uint32_t wsel, uint4* __restrict__ out, int* __restrict__ status)
{
	extern __shared__ __align__(16) unsigned char mw_smem[];
	unsigned long long* rv = reinterpret_cast<unsigned long long*>(mw_smem);     // [MJW_CAP]
	uint32_t* start = reinterpret_cast<uint32_t*>(rv + MJW_CAP);                // [MJ_LOCAL + 1]
	uint32_t* fill = start + MJ_LOCAL + 1;                                       // [MJ_LOCAL]
	uint32_t* wsum = fill + MJ_LOCAL;                                            // [MJW_THREADS / 32]
	const uint32_t b = blockIdx.x, tid = threadIdx.x;
	const uint64_t r0 = roffs[b], r1 = roffs[b + 1], s0 = soffs[b], s1 = soffs[b + 1];
	if (r1 - r0 > MJW_CAP) {             // the host checked every bucket; never taken
		if (tid == 0) pg_set_status(status, PG_ERR_UNSUPPORTED);
		return;
	}
	const unsigned long long kbase = (unsigned long long) kmin;
	for (uint32_t k = tid; k < MJ_LOCAL; k += MJW_THREADS) { start[k] = 0; fill[k] = 0; }
	__syncthreads();
	// Build side: per-key counts, their exclusive scan (run starts), then the
	// packed values scattered into their key's run.
	for (uint64_t i = r0 + tid; i < r1; i += MJW_THREADS) {
		const uint4 t = R[i];
		const unsigned long long key = ((unsigned long long) mjw_word(t, rkw + 1) << 32) | mjw_word(t, rkw);
		atomicAdd(&start[(key - kbase) & (MJ_LOCAL - 1)], 1u);
	}
	__syncthreads();
	{
		constexpr uint32_t PER = MJ_LOCAL / MJW_THREADS;        // 4 entries per thread
		uint32_t v[PER], run = 0;
		#pragma unroll
		for (uint32_t j = 0; j < PER; ++j) { v[j] = start[tid * PER + j]; run += v[j]; }
		uint32_t total;
		uint32_t base = mjw_block_scan(run, wsum, &total);
		#pragma unroll
		for (uint32_t j = 0; j < PER; ++j) { start[tid * PER + j] = base; base += v[j]; }
		if (tid == 0) start[MJ_LOCAL] = total;
	}
	__syncthreads();
	for (uint64_t i = r0 + tid; i < r1; i += MJW_THREADS) {
		const uint4 t = R[i];
		const unsigned long long key = ((unsigned long long) mjw_word(t, rkw + 1) << 32) | mjw_word(t, rkw);
		const uint32_t k = (uint32_t) ((key - kbase) & (MJ_LOCAL - 1));
		const uint32_t pos = start[k] + atomicAdd(&fill[k], 1u);
		unsigned long long pv = 0;
		if (bp.n > 0) pv = mjw_word(t, bp.roff[0]);
		if (bp.n > 1) pv |= (unsigned long long) mjw_word(t, bp.roff[1]) << 32;
		rv[pos] = pv;
	}
	__syncthreads();
	// Probe side in chunks of MJW_THREADS tuples, the next chunk's tuples
	// loaded while the current one is written. Tuple i of a chunk makes m_i
	// rows (one per build tuple of its key) at its scanned offset; the rows are
	// written load-balanced, thread j of the CTA taking the chunk's rows j,
	// j + MJW_THREADS, ..., so a warp stores 32 consecutive rows whatever the
	// duplicates. A row finds its probe tuple by binary search over the
	// offsets, which reuse the fill counters' shared memory (dead after the
	// build side).
	uint32_t* coff = fill;                                                       // [MJW_THREADS]
	uint32_t* crs = fill + MJW_THREADS;                                          // [MJW_THREADS]
	const uint32_t w0 = wsel & 15, w1 = (wsel >> 4) & 15, w2 = (wsel >> 8) & 15, w3 = (wsel >> 12) & 15;
	uint64_t row = bucket_off[b];
	uint4 tn = make_uint4(0, 0, 0, 0);
	if (s0 + tid < s1) tn = S[s0 + tid];
	for (uint64_t c0 = s0; c0 < s1; c0 += MJW_THREADS) {
		const uint4 t = tn;
		const uint64_t i = c0 + tid;
		if (i + MJW_THREADS < s1) tn = S[i + MJW_THREADS];
		uint32_t m = 0, rs = 0;
		if (i < s1) {
			const unsigned long long key = ((unsigned long long) mjw_word(t, skw + 1) << 32) | mjw_word(t, skw);
			const uint32_t k = (uint32_t) ((key - kbase) & (MJ_LOCAL - 1));
			rs = start[k];
			m = start[k + 1] - rs;
		}
		uint32_t total;
		// The scan's barriers also order this chunk's offset writes after
		// every thread's reads of the previous chunk's offsets.
		const uint32_t off = mjw_block_scan(m, wsum, &total);
		coff[tid] = off;
		crs[tid] = rs;
		__syncthreads();
		for (uint32_t j = tid; j < total; j += MJW_THREADS) {
			uint32_t x = 0;                  // the last tuple whose offset is <= j (it has m > 0)
			#pragma unroll
			for (uint32_t step = MJW_THREADS / 2; step; step >>= 1)
				if (coff[x + step] <= j) x += step;
			const unsigned long long v = rv[crs[x] + (j - coff[x])];
			const uint4 p = S[c0 + x];
			out[row + j] = make_uint4(mjw_pick(p, v, w0), mjw_pick(p, v, w1), mjw_pick(p, v, w2), mjw_pick(p, v, w3));
		}
		row += total;
	}
}

// Largest build-side bucket (roffs[b + 1] - roffs[b]) into *mx.
__global__ void k_mj_max_bucket(const uint64_t* __restrict__ offs, uint32_t B, unsigned long long* __restrict__ mx)
{
	unsigned long long m = 0;
	for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < B; b += gridDim.x * blockDim.x)
		m = max(m, (unsigned long long) (offs[b + 1] - offs[b]));
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_down_sync(0xffffffffu, m, o));
	if ((threadIdx.x & 31) == 0 && m) atomicMax(mx, m);
}

// Word selector (4 bits per output word: 0-3 probe tuple word, 4-5 packed
// build word) and packed build words of the 16-byte output rows of the
// bucketed materialising join; false when the layout is not one it takes:
// 16-byte tuples with 8-byte keys on both sides, 16-byte rows whose build
// words other than the key (taken from the probe tuple's equal key) fit 8 bytes.
static bool mj_bucket_rows_fit(const pg_rel* R, const pg_rel* S, const MjCols& pc, uint32_t* wsel, MjPack* bp)
{
	if (R->width != 16 || S->width != 16 || R->key_bytes != 8 || S->key_bytes != 8 || (R->key_off & 7) ||
			(S->key_off & 7) || pc.ow_words != 4 ||
			(reinterpret_cast<uintptr_t>(R->data) & 15) || (reinterpret_cast<uintptr_t>(S->data) & 15))
		return false;
	bp->n = 0; bp->roff[0] = bp->roff[1] = 0;
	*wsel = 0;
	uint32_t o = 0;
	for (int c = 0; c < pc.n; ++c)
		for (uint32_t j = 0; j < pc.words[c]; ++j, ++o) {
			const uint32_t byte = pc.off[c] + 4 * j;
			uint32_t sel;
			if (pc.side[c]) {
				sel = byte / 4;
			} else if (byte >= R->key_off && byte < R->key_off + 8) {
				sel = (S->key_off + (byte - R->key_off)) / 4;
			} else {
				int p = -1;
				for (int q = 0; q < bp->n; ++q) if (bp->roff[q] == byte / 4) p = q;
				if (p < 0) {
					if (bp->n == 2) return false;
					p = bp->n;
					bp->roff[bp->n++] = (uint8_t) (byte / 4);
				}
				sel = 4 + (uint32_t) p;
			}
			*wsel |= sel << (4 * o);
		}
	return true;
}

// Joins over key buckets when the key span is 2^13..2^24 values: both sides
// partitioned on the key bits above the low 12, then each bucket pair in
// shared memory. Without `materialize` the per-key counts give the count and
// sum (MjCols sum column); with it, the rows are written (16-byte layouts
// that mj_bucket_rows_fit takes, every bucket's build side within MJW_CAP
// tuples). *handled = false (nothing produced) when the case is not one it
// takes: the caller then sorts.
static int mj_bucket_join(pg_ctx* ctx, cudaStream_t s, const pg_rel* R, const pg_rel* S, const MjCols& pc,
		int sum_col, int flags, void* out, uint64_t out_capacity, pg_join_result* res, bool* handled,
		bool* r_sorted, bool* s_sorted)
{
	*handled = false;
	*r_sorted = *s_sorted = false;
	const bool materialize = (flags & PG_JOIN_MATERIALIZE) != 0;
	uint32_t wsel = 0;
	MjPack bp;
	const bool rows_fit = mj_bucket_rows_fit(R, S, pc, &wsel, &bp) && !(reinterpret_cast<uintptr_t>(out) & 15);
	int rc;
	// [key min, key max, count, sum, largest build bucket, R unsorted, S unsorted]
	unsigned long long* mm = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &mm, 64))) return rc;
	const unsigned long long init[8] = {~0ull, 0ull, 0ull, 0ull, 0ull, 0ull, 0ull, 0ull};
	PG_CUDA(ctx, cudaMemcpyAsync(mm, init, 64, cudaMemcpyHostToDevice, s));
	for (int side = 0; side < 2; ++side) {
		const pg_rel* r = side ? S : R;
		const bool check = (flags & (side ? PG_JOIN_PROBE_SORTED : PG_JOIN_BUILD_SORTED)) != 0;
		const int blocks = (int) std::min<uint64_t>(pg_div_up(r->n, 256), (uint64_t) ctx->sm_count * 8);
		k_mj_minmax<<<blocks, 256, 0, s>>>((const char*) r->data, r->n, r->width, r->key_off, r->key_bytes, mm,
				check ? mm + 5 + side : nullptr);
		PG_LAUNCHED(ctx);
	}
	unsigned long long h[8];
	PG_CUDA(ctx, cudaMemcpyAsync(h, mm, 64, cudaMemcpyDeviceToHost, s));
	PG_CUDA(ctx, cudaStreamSynchronize(s));
	// A side confirmed sorted skips its sort (here: its bucket partition).
	*r_sorted = (flags & PG_JOIN_BUILD_SORTED) && !h[5];
	*s_sorted = (flags & PG_JOIN_PROBE_SORTED) && !h[6];
	if (materialize && !rows_fit) { pg_free_async(ctx, s, mm); return PG_OK; }
	const unsigned long long span = h[1] - h[0];
	const int bits = span == 0 ? 0 : 64 - __builtin_clzll(span);
	if (bits <= (int) MJ_LOCAL_BITS || bits > (int) MJ_LOCAL_BITS + 12) { pg_free_async(ctx, s, mm); return PG_OK; }
	const long long kmin = (long long) (h[0] ^ (1ull << 63));
	const int hb = bits - MJ_LOCAL_BITS;
	const uint32_t B = 1u << hb;
	// Stable radix passes over the bucket bits (one of up to 8 bits, or two
	// halves of at most 6: the fast partition shapes), then the bucket
	// bounds by binary search.
	const int npass = hb <= 8 ? 1 : 2;
	const int d0 = npass == 1 ? hb : hb / 2;
	char *pR = nullptr, *pS = nullptr, *tmp = nullptr;
	uint64_t *oR = nullptr, *oS = nullptr, *brows = nullptr;
	auto release = [&]() {
		for (void* p : {(void*) pR, (void*) pS, (void*) tmp, (void*) oR, (void*) oS, (void*) brows, (void*) mm})
			pg_free_async(ctx, s, p);
	};
	if (!*r_sorted && (rc = pg_alloc_async(ctx, s, (void**) &pR, R->n * R->width))) return rc;
	if (!*s_sorted && (rc = pg_alloc_async(ctx, s, (void**) &pS, S->n * S->width))) return rc;
	if (npass == 2 && !(*r_sorted && *s_sorted) &&
			(rc = pg_alloc_async(ctx, s, (void**) &tmp, std::max(R->n * R->width, S->n * S->width)))) return rc;
	if ((rc = pg_alloc_async(ctx, s, (void**) &oR, (B + 1) * 8))) return rc;
	if ((rc = pg_alloc_async(ctx, s, (void**) &oS, (B + 1) * 8))) return rc;
	if (materialize && (rc = pg_alloc_async(ctx, s, (void**) &brows, (B + 1) * 8))) return rc;
	const char* bR = *r_sorted ? (const char*) R->data : pR;   // each side in bucket order
	const char* bS = *s_sorted ? (const char*) S->data : pS;
	for (int side = 0; side < 2; ++side) {
		const pg_rel* in = side ? S : R;
		char* dst = side ? pS : pR;
		pg_rel cur = *in;
		const bool sorted = side ? *s_sorted : *r_sorted;
		for (int p = 0; p < npass && !sorted; ++p) {
			const int d = p == 0 ? d0 : hb - d0;
			pg_hashfn f;
			f.fn = PG_FN_PARAMMODULO;
			f.skipbits = MJ_LOCAL_BITS + (p == 0 ? 0 : d0);
			f.k = (int64_t) ((1u << d) - 1) << f.skipbits;
			f.min = kmin;
			f.max = 0; f.bucketrange = 0;
			f.nbuckets = 1u << d;
			char* o = (npass == 2 && p == 0) ? tmp : dst;
			if ((rc = pg_partition_fn(ctx, s, &cur, f, o, nullptr))) return rc;
			cur.data = o;
		}
		k_mj_bounds<<<(B + 256) / 256, 256, 0, s>>>(side ? bS : bR, in->n, in->width, in->key_off, in->key_bytes,
				kmin, B, side ? oS : oR);
		PG_LAUNCHED(ctx);
	}
	PG_CUDA(ctx, cudaMemsetAsync(mm + 2, 0, 24, s));
	const int sum_side = sum_col < 0 ? -1 : (int) pc.side[sum_col];
	const size_t smem = MJ_LOCAL * (8 + 4 + 4);
	PG_CUDA(ctx, cudaFuncSetAttribute(k_mj_bucket_join, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
	k_mj_bucket_join<<<B, 256, smem, s>>>(bR, oR, R->width, R->key_off, R->key_bytes, bS, oS, S->width, S->key_off,
			S->key_bytes, kmin, sum_side, sum_col >= 0 ? pc.off[sum_col] : 0, sum_col >= 0 ? pc.words[sum_col] : 0,
			mm + 2, brows);
	PG_LAUNCHED(ctx);
	if (materialize) {
		if ((rc = pg_scan_u64(ctx, s, brows, B, nullptr))) { release(); return rc; }
		k_mj_max_bucket<<<(B + 255) / 256, 256, 0, s>>>(oR, B, mm + 4);
		PG_LAUNCHED(ctx);
	}
	unsigned long long o[3];
	PG_CUDA(ctx, cudaMemcpyAsync(o, mm + 2, 24, cudaMemcpyDeviceToHost, s));
	if ((rc = pg_check_status(ctx, s, "pg_mpsm_join"))) { release(); return rc; }
	if (materialize && o[2] > MJW_CAP) { release(); return PG_OK; }     // a bucket too large: sort instead
	res->n_out = o[0];
	res->sum = (int64_t) o[1];
	*handled = true;
	if (materialize && o[0]) {
		if (o[0] > out_capacity) {
			release();
			return pg_fail(ctx, PG_ERR_OUTPUT_FULL, "pg_mpsm_join: output capacity too small");
		}
		const size_t wsmem = MJW_CAP * 8 + (2 * MJ_LOCAL + 1) * 4 + (MJW_THREADS / 32) * 4;
		PG_CUDA(ctx, cudaFuncSetAttribute(k_mj_bucket_write, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) wsmem));
		k_mj_bucket_write<<<B, MJW_THREADS, wsmem, s>>>(reinterpret_cast<const uint4*>(bR), oR, R->key_off / 4, bp,
				reinterpret_cast<const uint4*>(bS), oS, S->key_off / 4, kmin, brows, wsel,
				reinterpret_cast<uint4*>(out), ctx->d_status);
		PG_LAUNCHED(ctx);
		rc = pg_check_status(ctx, s, "pg_mpsm_join");
	}
	release();
	return rc;
}

extern "C" int pg_mpsm_join(pg_ctx* ctx, pg_stream stream, const pg_rel* R, const pg_rel* S,
		const pg_col* proj, int nproj, void* out, uint64_t out_capacity,
		int flags, int sum_col, pg_join_result* res)
{
	if (!ctx || !R || !S || !res) return pg_fail(ctx, PG_ERR_ARG, "pg_mpsm_join: null argument");
	for (const pg_rel* r : {R, S}) {
		if (r->n && !r->data) return pg_fail(ctx, PG_ERR_ARG, "pg_mpsm_join: null data");
		if (r->width == 0 || (r->width & 3) || (r->key_bytes != 4 && r->key_bytes != 8) ||
				(r->key_off & 3) || r->key_off + r->key_bytes > r->width)
			return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_mpsm_join: 4-byte-aligned tuples with an int or long key");
	}
	if (nproj < 0 || nproj > MJ_MAX_COLS) return pg_fail(ctx, PG_ERR_ARG, "pg_mpsm_join: 0..16 columns");
	MjCols pc; pc.n = nproj; pc.ow_words = 0;
	for (int i = 0; i < nproj; ++i) {
		const pg_col& c = proj[i];
		uint32_t w = c.side ? S->width : R->width;
		if (c.side > 1 || (c.bytes != 4 && c.bytes != 8) || (c.off & 3) || c.off + c.bytes > w)
			return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_mpsm_join: projected columns must be 4/8 bytes, aligned");
		pc.side[i] = (uint8_t) c.side; pc.off[i] = (uint16_t) c.off; pc.words[i] = (uint8_t) (c.bytes / 4);
		pc.ow_words += c.bytes / 4;
	}
	if (sum_col >= nproj) return pg_fail(ctx, PG_ERR_ARG, "pg_mpsm_join: sum_col out of range");
	if (!(flags & PG_JOIN_SUM)) sum_col = -1;
	const bool materialize = (flags & PG_JOIN_MATERIALIZE) != 0;
	res->n_out = 0; res->sum = 0;
	if (R->n == 0 || S->n == 0) return PG_OK;
	cudaStream_t s = (cudaStream_t) stream;
	int rc;
	bool r_sorted = false, s_sorted = false;   // confirmed on the device
	if (R->n < (1ull << 32) && S->n < (1ull << 32)) {
		bool handled = false;
		if ((rc = mj_bucket_join(ctx, s, R, S, pc, sum_col, flags, out, out_capacity, res, &handled, &r_sorted,
				&s_sorted))) return rc;
		if (handled) return PG_OK;
	}
	// A sorted 16-byte tuple keyed at offset 0 is its own sorted record array.
	pg_rec *rr = nullptr, *sr = nullptr;
	const bool r_own = !(r_sorted && pg_sort_mode(R) == 0 && !(reinterpret_cast<uintptr_t>(R->data) & 15));
	const bool s_own = !(s_sorted && pg_sort_mode(S) == 0 && !(reinterpret_cast<uintptr_t>(S->data) & 15));
	if (r_own) { if ((rc = pg_sort_records(ctx, s, R, &rr))) return rc; }
	else rr = (pg_rec*) R->data;
	if (s_own) { if ((rc = pg_sort_records(ctx, s, S, &sr))) return rc; }
	else sr = (pg_rec*) S->data;
	MjSide RS{rr, (const char*) R->data, R->width, R->key_off, pg_sort_mode(R), nullptr, 0};
	MjSide SS{sr, (const char*) S->data, S->width, S->key_off, pg_sort_mode(S), nullptr, 0};
	uint64_t *rst = nullptr, *sst = nullptr;
	long long *rk = nullptr, *sk = nullptr;
	if ((rc = mj_runs(ctx, s, rr, R->n, &rst, &rk, &RS.nruns))) return rc;
	if ((rc = mj_runs(ctx, s, sr, S->n, &sst, &sk, &SS.nruns))) return rc;
	RS.run_start = rst; SS.run_start = sst;
	uint64_t *counts = nullptr, *match = nullptr;
	unsigned long long* acc = nullptr;  // [total, sum]
	if ((rc = pg_alloc_async(ctx, s, (void**) &counts, (RS.nruns + 1) * 8))) return rc;
	if ((rc = pg_alloc_async(ctx, s, (void**) &match, (RS.nruns + 1) * 8))) return rc;
	if ((rc = pg_alloc_async(ctx, s, (void**) &acc, 16))) return rc;
	PG_CUDA(ctx, cudaMemsetAsync(acc, 0, 16, s));
	// One warp per MJ_WARP_RUNS build runs, 8 warps per CTA.
	int blocks = (int) std::min<uint64_t>(pg_div_up(pg_div_up(RS.nruns, MJ_WARP_RUNS), 8), (uint64_t) ctx->sm_count * 16);
	k_match_runs<<<std::max(blocks, 1), 256, 0, s>>>(RS, SS, rk, sk, pc, sum_col, counts, match, acc + 1);
	PG_LAUNCHED(ctx);
	if ((rc = pg_scan_u64(ctx, s, counts, RS.nruns, (uint64_t*) acc))) return rc;
	unsigned long long h[2];
	PG_CUDA(ctx, cudaMemcpyAsync(h, acc, 16, cudaMemcpyDeviceToHost, s));
	if ((rc = pg_check_status(ctx, s, "pg_mpsm_join"))) return rc;
	res->n_out = h[0];
	res->sum = (int64_t) h[1];
	if (materialize && res->n_out) {
		if (res->n_out > out_capacity) {
			rc = pg_fail(ctx, PG_ERR_OUTPUT_FULL, "pg_mpsm_join: output capacity too small");
		} else {
			PG_CUDA(ctx, cudaMemcpyAsync(counts + RS.nruns, &res->n_out, 8, cudaMemcpyHostToDevice, s));
			int wb = (int) std::min<uint64_t>(pg_div_up(pg_div_up(res->n_out, MJ_PER_THREAD), 256), (uint64_t) ctx->sm_count * 16);
			k_mj_write<<<wb, 256, 0, s>>>(RS, SS, pc, counts, match, res->n_out, (char*) out);
			PG_LAUNCHED(ctx);
			rc = pg_check_status(ctx, s, "pg_mpsm_join");
		}
	}
	for (void* p : {r_own ? (void*) rr : nullptr, s_own ? (void*) sr : nullptr, (void*) rst, (void*) sst, (void*) rk,
			(void*) sk, (void*) counts, (void*) match, (void*) acc})
		pg_free_async(ctx, s, p);
	return rc;
}
