// Page sort on sm_103a: bitonic tile sort in shared memory + merge-path merges.
//
// Replaces TupleBuffer::sort<KeyT> (util/buffer.inl:135-292, std::sort on the
// key at keyoffset, reached through sortAllInPage, operators/join.cpp:893-912)
// and the SSE bitonic block sort (util/bitonicsort.cpp:371-443), which sorts
// 4096-record cache blocks with a bitonic network and then merges blocks
// pairwise. The same structure here: a CTA stages a 4096-tuple page in shared
// memory (bulk copy, cp.async.bulk + mbarrier), sorts (key, position) pairs
// with a bitonic network, and writes the page in key order; then log2(n/4096)
// merge passes, each CTA producing 2048 outputs of a run pair located by a
// merge-path binary search (Odeh et al., "Merge Path", 2012).
//
// Keys spanning at most 2^32 values take an LSD radix path instead (see
// radix_sort below). Tuples travel as 16-byte records {int64 key, uint64 val}. A 16-byte tuple
// with an 8-byte key is its own record (the key half first); any other layout
// sorts (widened key, row index) records and gathers rows at the end. Ties are
// left in unspecified order, as std::sort leaves them. Unlike the reference's
// bitonic path (asserting power-of-two sizes above 4096 records,
// util/buffer.cpp:101-104) any n is accepted, including n = 4096.
#include "pg_internal.cuh"
#include "pg_sort.cuh"
#include <algorithm>

#define TS_TILE 4096
#define TS_THREADS 512
#define MG_THREADS 256
#define MG_ITEMS 8
#define MG_CHUNK (MG_THREADS * MG_ITEMS)

// Mode: 0 = 16-byte tuple, key at 0; 1 = 16-byte tuple, key at 8; 2 = index records.
__global__ void __launch_bounds__(TS_THREADS)
k_tile_sort(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t koff, uint32_t kbytes,
		int mode, pg_rec* __restrict__ out, bool bulk_ok, int* __restrict__ status)
{
	extern __shared__ __align__(128) unsigned char sm[];
	pg_rec* rec = reinterpret_cast<pg_rec*>(sm);                        // [TS_TILE]
	long long* key = reinterpret_cast<long long*>(rec + TS_TILE);      // [TS_TILE]
	uint16_t* pos = reinterpret_cast<uint16_t*>(key + TS_TILE);        // [TS_TILE]
	__shared__ __align__(8) uint64_t bar;
	const int tid = threadIdx.x;
	const uint64_t base = (uint64_t) blockIdx.x * TS_TILE;
	const uint32_t rows = (uint32_t) pg_min64(TS_TILE, n - base);

	if (mode != 2) {
		const uint32_t bytes = rows * 16;
		if (bulk_ok) {
			if (tid == 0) {
				pg_mbar_init(&bar, 1);
				pg_fence_mbar_init();
				pg_mbar_expect_tx(&bar, bytes);
				pg_bulk_g2s(rec, in + base * 16, bytes, &bar);
			}
			__syncthreads();
			// A wait past the context's limit records PG_ERR_TIMEOUT and then
			// drains the copy; only a copy that never lands ends the block.
			if (!pg_mbar_wait_timed(&bar, 0, pg_spin_knob(status), status)) return;
		} else {
			const uint4* src = reinterpret_cast<const uint4*>(in + base * 16);
			for (uint32_t i = tid; i < rows; i += blockDim.x) reinterpret_cast<uint4*>(rec)[i] = src[i];
		}
		__syncthreads();
		if (mode == 1)
			for (uint32_t i = tid; i < rows; i += blockDim.x) {
				pg_rec r = rec[i];
				rec[i].key = (long long) r.val; rec[i].val = (unsigned long long) r.key;
			}
	} else {
		for (uint32_t i = tid; i < rows; i += blockDim.x) {
			rec[i].key = pg_load_key(in + (base + i) * W + koff, kbytes);
			rec[i].val = base + i;
		}
	}
	__syncthreads();
	for (uint32_t i = tid; i < TS_TILE; i += blockDim.x) {
		key[i] = i < rows ? rec[i].key : 0;
		pos[i] = (uint16_t) i;
	}
	__syncthreads();
	// Bitonic network over (key, pad) with pad = position >= rows, so padding
	// sorts after every real tuple whatever its key.
	for (uint32_t k = 2; k <= TS_TILE; k <<= 1) {
		for (uint32_t j = k >> 1; j > 0; j >>= 1) {
			for (uint32_t t = tid; t < TS_TILE / 2; t += blockDim.x) {
				uint32_t i = 2 * t - (t & (j - 1));
				uint32_t l = i + j;
				long long ki = key[i], kl = key[l];
				uint16_t pi = pos[i], pl = pos[l];
				bool padi = pi >= rows, padl = pl >= rows;
				bool gt = (padi != padl) ? padi : (ki > kl);
				bool asc = (i & k) == 0;
				if (gt == asc) { key[i] = kl; key[l] = ki; pos[i] = pl; pos[l] = pi; }
			}
			__syncthreads();
		}
	}
	for (uint32_t i = tid; i < rows; i += blockDim.x) out[base + i] = rec[pos[i]];
}

__device__ __forceinline__ uint64_t merge_path(const pg_rec* A, uint64_t la, const pg_rec* B, uint64_t lb, uint64_t d)
{
	uint64_t lo = d > lb ? d - lb : 0, hi = d < la ? d : la;
	while (lo < hi) {
		uint64_t mid = (lo + hi) >> 1;
		if (A[mid].key <= B[d - 1 - mid].key) lo = mid + 1; else hi = mid;
	}
	return lo;
}

__global__ void __launch_bounds__(MG_THREADS)
k_merge_pass(const pg_rec* __restrict__ src, pg_rec* __restrict__ dst, uint64_t n, uint64_t L)
{
	__shared__ pg_rec sA[MG_CHUNK];
	__shared__ uint64_t split[2];
	const uint64_t o0 = (uint64_t) blockIdx.x * MG_CHUNK;
	if (o0 >= n) return;
	const uint64_t p0 = o0 / (2 * L) * (2 * L);
	const pg_rec* A = src + p0;
	const uint64_t la = pg_min64(L, n - p0);
	const pg_rec* B = A + la;
	const uint64_t lb = (n - p0 > L) ? pg_min64(L, n - p0 - L) : 0;
	const uint64_t d0 = o0 - p0, d1 = pg_min64(d0 + MG_CHUNK, la + lb);
	if (threadIdx.x < 2) split[threadIdx.x] = merge_path(A, la, B, lb, threadIdx.x ? d1 : d0);
	__syncthreads();
	const uint64_t a0 = split[0], a1 = split[1];
	const uint64_t b0 = d0 - a0, b1 = d1 - a1;
	const uint32_t na = (uint32_t) (a1 - a0), nb = (uint32_t) (b1 - b0);
	// Stage both slices back to back: [A slice][B slice].
	for (uint32_t i = threadIdx.x; i < na + nb; i += blockDim.x)
		sA[i] = i < na ? A[a0 + i] : B[b0 + i - na];
	__syncthreads();
	const pg_rec* xa = sA;
	const pg_rec* xb = sA + na;
	const uint32_t dt = threadIdx.x * MG_ITEMS;
	const uint32_t total = na + nb;
	if (dt >= total) return;
	// Split of this thread's diagonal inside the staged slices.
	uint32_t lo = dt > nb ? dt - nb : 0, hi = dt < na ? dt : na;
	while (lo < hi) {
		uint32_t mid = (lo + hi) >> 1;
		if (xa[mid].key <= xb[dt - 1 - mid].key) lo = mid + 1; else hi = mid;
	}
	uint32_t i = lo, j = dt - lo;
	const uint32_t cnt = pg_min32(MG_ITEMS, total - dt);
	pg_rec* o = dst + o0 + dt;
	for (uint32_t q = 0; q < cnt; ++q) {
		bool takeA = j >= nb || (i < na && xa[i].key <= xb[j].key);
		o[q] = takeA ? xa[i++] : xb[j++];
	}
}

__global__ void k_records_to_tuples(const pg_rec* __restrict__ rec, uint64_t n, int mode,
		const char* __restrict__ in, uint32_t W, char* __restrict__ out)
{
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
			i += (uint64_t) gridDim.x * blockDim.x) {
		pg_rec r = rec[i];
		if (mode == 0) reinterpret_cast<pg_rec*>(out)[i] = r;
		else if (mode == 1) {
			pg_rec t; t.key = (long long) r.val; t.val = (unsigned long long) r.key;
			reinterpret_cast<pg_rec*>(out)[i] = t;
		} else {
			const uint32_t* s = reinterpret_cast<const uint32_t*>(in + r.val * W);
			uint32_t* d = reinterpret_cast<uint32_t*>(out + i * W);
			for (uint32_t w = 0; w < W / 4; ++w) d[w] = s[w];
		}
	}
}

// ---------------------------------------------------------------------------
// LSD radix path: when the keys span at most 2^32 values, ceil(bits/d) stable
// 2^d-way partitions on successive d-bit digits of (key - min) (d = 8, or the
// PG_TUNE_RADIX_BITS knob, 4..12) sort the
// tuples (pg_partition.cu; each pass reads and writes the relation once). This
// is ParameterizedModuloValueHasher::generate's multi-pass radix split
// (hash.cpp:237-267) driven to completion. Ties keep input order.
// ---------------------------------------------------------------------------
__global__ void k_sort_minmax(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t koff,
		uint32_t kbytes, unsigned long long* __restrict__ mm)
{
	unsigned long long lo = ~0ull, hi = 0;
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
			i += (uint64_t) gridDim.x * blockDim.x) {
		const unsigned long long u = (unsigned long long) pg_load_key(in + i * W + koff, kbytes) ^ (1ull << 63);
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

// (key, other half) or (key, row index) records for layouts other than a
// 16-byte tuple keyed at offset 0.
__global__ void k_make_records(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t koff,
		uint32_t kbytes, int mode, pg_rec* __restrict__ out)
{
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
			i += (uint64_t) gridDim.x * blockDim.x) {
		pg_rec r;
		if (mode == 1) {
			const pg_rec t = reinterpret_cast<const pg_rec*>(in)[i];
			r.key = (long long) t.val; r.val = (unsigned long long) t.key;
		} else {
			r.key = pg_load_key(in + i * W + koff, kbytes);
			r.val = i;
		}
		out[i] = r;
	}
}

// Sorts `in` into `out` by radix passes when the key span allows; returns
// PG_OK with *done = false (nothing queued) when it does not. `tmp` holds n
// tuples of scratch.
static int radix_sort(pg_ctx* ctx, cudaStream_t s, const pg_rel* in, void* out, void* tmp, bool* done)
{
	*done = false;
	const uint64_t n = in->n;
	if (n == 0 || n >= (1ull << 32)) return PG_OK;
	int rc;
	unsigned long long* mm = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &mm, 16))) return rc;
	const unsigned long long init[2] = {~0ull, 0ull};
	PG_CUDA(ctx, cudaMemcpyAsync(mm, init, 16, cudaMemcpyHostToDevice, s));
	const int blocks = (int) std::min<uint64_t>(pg_div_up(n, 256), (uint64_t) ctx->sm_count * 8);
	k_sort_minmax<<<blocks, 256, 0, s>>>((const char*) in->data, n, in->width, in->key_off, in->key_bytes, mm);
	PG_LAUNCHED(ctx);
	unsigned long long h[2];
	PG_CUDA(ctx, cudaMemcpyAsync(h, mm, 16, cudaMemcpyDeviceToHost, s));
	PG_CUDA(ctx, cudaStreamSynchronize(s));
	pg_free_async(ctx, s, mm);
	const unsigned long long span = h[1] - h[0];
	const int bits = span == 0 ? 0 : 64 - __builtin_clzll(span);
	// LSD radix over the bits of key - min while they fit 63 bits (the digit
	// function masks a signed difference). Bitonic tiles and merge-path
	// merges instead for wider spans, and for small inputs whose span needs
	// more than four 8-bit passes: there the few merge passes cost less than
	// the radix passes (a histogram read and a scatter each).
	const int64_t path = ctx->tune[PG_TUNE_SORT_PATH];
	if (path == 2 || bits > 63) return PG_OK;
	if (path == 0 && bits > 32 && n <= (1ull << 18)) return PG_OK;
	const long long kmin = (long long) (h[0] ^ (1ull << 63));
	if (bits == 0) {   // one key value: already sorted
		PG_CUDA(ctx, cudaMemcpyAsync(out, in->data, n * in->width, cudaMemcpyDeviceToDevice, s));
		*done = true;
		return PG_OK;
	}
	const int64_t tb = ctx->tune[PG_TUNE_RADIX_BITS];
	const int digit = tb >= 4 && tb <= 12 ? (int) tb : 8;
	const int passes = (bits + digit - 1) / digit;
	pg_rel cur = *in;
	for (int p = 0; p < passes; ++p) {
		pg_hashfn f;
		f.fn = PG_FN_PARAMMODULO;
		f.skipbits = digit * p;
		f.k = (int64_t) ((1u << digit) - 1) << f.skipbits;
		f.min = kmin;
		f.max = 0; f.bucketrange = 0;
		f.nbuckets = 1u << digit;
		void* dst = ((passes - 1 - p) % 2 == 0) ? out : tmp;
		if ((rc = pg_partition_fn(ctx, s, &cur, f, dst, nullptr))) return rc;
		cur.data = dst;
	}
	*done = true;
	return PG_OK;
}

int pg_sort_mode(const pg_rel* r)
{
	if (r->width == 16 && r->key_bytes == 8 && r->key_off == 0) return 0;
	if (r->width == 16 && r->key_bytes == 8 && r->key_off == 8) return 1;
	return 2;
}

// Sorts `in` into records; *recs receives a pool allocation of n records
// (caller frees with pg_free_async on stream s).
int pg_sort_records(pg_ctx* ctx, cudaStream_t s, const pg_rel* in, pg_rec** recs)
{
	const uint64_t n = in->n;
	int rc;
	const int mode = pg_sort_mode(in);
	pg_rec *a = nullptr, *b = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &a, n * sizeof(pg_rec)))) return rc;
	if (n == 0) { *recs = a; return PG_OK; }
	{
		// Radix path: sort 16-byte records (the tuples themselves when the
		// layout is a 16-byte tuple keyed at 0).
		pg_rec* src = nullptr;
		pg_rel r = *in;
		if (mode != 0) {
			if ((rc = pg_alloc_async(ctx, s, (void**) &src, n * sizeof(pg_rec)))) return rc;
			const int blocks = (int) std::min<uint64_t>(pg_div_up(n, 256), (uint64_t) ctx->sm_count * 16);
			k_make_records<<<blocks, 256, 0, s>>>((const char*) in->data, n, in->width, in->key_off,
					in->key_bytes, mode, src);
			PG_LAUNCHED(ctx);
			r.data = src; r.width = 16; r.key_off = 0; r.key_bytes = 8;
		}
		if ((rc = pg_alloc_async(ctx, s, (void**) &b, n * sizeof(pg_rec)))) return rc;
		bool done = false;
		if ((rc = radix_sort(ctx, s, &r, a, b, &done))) return rc;
		pg_free_async(ctx, s, b);
		b = nullptr;
		if (src) pg_free_async(ctx, s, src);
		if (done) { *recs = a; return PG_OK; }
	}
	const uint64_t tiles = pg_div_up(n, TS_TILE);
	const size_t smem = TS_TILE * (sizeof(pg_rec) + 8 + 2);
	PG_CUDA(ctx, cudaFuncSetAttribute(k_tile_sort, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem));
	const bool bulk_ok = mode != 2 && (reinterpret_cast<uintptr_t>(in->data) & 15) == 0;
	k_tile_sort<<<(unsigned) tiles, TS_THREADS, smem, s>>>((const char*) in->data, n, in->width, in->key_off,
			in->key_bytes, mode, a, bulk_ok, ctx->d_status);
	PG_LAUNCHED(ctx);
	if (n > TS_TILE) {
		if ((rc = pg_alloc_async(ctx, s, (void**) &b, n * sizeof(pg_rec)))) return rc;
		const unsigned blocks = (unsigned) pg_div_up(n, MG_CHUNK);
		for (uint64_t L = TS_TILE; L < n; L <<= 1) {
			k_merge_pass<<<blocks, MG_THREADS, 0, s>>>(a, b, n, L);
			PG_LAUNCHED(ctx);
			std::swap(a, b);
		}
		pg_free_async(ctx, s, b);
	}
	*recs = a;
	return PG_OK;
}

extern "C" int pg_sort_pages(pg_ctx* ctx, pg_stream stream, const pg_rel* in, void* out)
{
	if (!ctx || !in) return pg_fail(ctx, PG_ERR_ARG, "pg_sort_pages: null argument");
	if (in->n && (!in->data || !out)) return pg_fail(ctx, PG_ERR_ARG, "pg_sort_pages: null data");
	if (in->width == 0 || (in->width & 3) || (in->key_bytes != 4 && in->key_bytes != 8) ||
			(in->key_off & 3) || in->key_off + in->key_bytes > in->width)
		return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_sort_pages: 4-byte-aligned tuples with an int or long key");
	if (in->data == out && in->n) return pg_fail(ctx, PG_ERR_ARG, "pg_sort_pages: output may not alias input");
	cudaStream_t s = (cudaStream_t) stream;
	if (in->n == 0) return PG_OK;
	pg_rec* recs = nullptr;
	int rc;
	{
		void* tmp = nullptr;
		if ((rc = pg_alloc_async(ctx, s, &tmp, in->n * in->width))) return rc;
		bool done = false;
		rc = radix_sort(ctx, s, in, out, tmp, &done);
		pg_free_async(ctx, s, tmp);
		if (rc) return rc;
		if (done) return pg_check_status(ctx, s, "pg_sort_pages");
	}
	if ((rc = pg_sort_records(ctx, s, in, &recs))) return rc;
	const int mode = pg_sort_mode(in);
	int blocks = (int) std::min<uint64_t>(pg_div_up(in->n, 256), (uint64_t) ctx->sm_count * 16);
	k_records_to_tuples<<<blocks, 256, 0, s>>>(recs, in->n, mode, (const char*) in->data, in->width, (char*) out);
	PG_LAUNCHED(ctx);
	pg_free_async(ctx, s, recs);
	return pg_check_status(ctx, s, "pg_sort_pages");
}

extern "C" int pg_partition_sort(pg_ctx* ctx, pg_stream stream, const pg_rel* data,
		const uint64_t* offsets_host, uint32_t nbuckets, void* scratch_out)
{
	if (!ctx || !data || !offsets_host || !scratch_out)
		return pg_fail(ctx, PG_ERR_ARG, "pg_partition_sort: null argument");
	cudaStream_t s = (cudaStream_t) stream;
	for (uint32_t b = 0; b < nbuckets; ++b) {
		pg_rel part = *data;
		part.data = (const char*) data->data + offsets_host[b] * data->width;
		part.n = offsets_host[b + 1] - offsets_host[b];
		if (part.n == 0) continue;
		int rc = pg_sort_pages(ctx, stream, &part, (char*) scratch_out + offsets_host[b] * data->width);
		if (rc) return rc;
	}
	PG_CUDA(ctx, cudaMemcpyAsync((void*) data->data, scratch_out, data->n * data->width, cudaMemcpyDeviceToDevice, s));
	return pg_check_status(ctx, s, "pg_partition_sort");
}
