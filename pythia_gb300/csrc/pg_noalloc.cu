// Hash join count/sum that allocates nothing.
//
// Some callers cannot allocate device memory while they run a query: a host
// that reserved the whole device for its own pool and forbids further
// cudaMalloc calls, a plugin sandbox with a fixed memory budget, or code that
// must not trigger allocator work (and its implicit synchronisation) on a
// latency-critical path. For them, pg_hashjoin_agg_noalloc computes what
// pg_hashjoin_build + pg_hashjoin_probe(PG_JOIN_COUNT | PG_JOIN_SUM) compute,
// with its hash table in one fixed array in device global memory that this
// file declares at file scope. The caller still passes inputs; the result
// comes back in a host struct.
//
// Limits and sharing:
//   * at most PG_NOALLOC_MAX_BUILD (524,288) build tuples; larger build sides
//     are rejected with PG_ERR_ARG. The array is 16 MiB of table plus a small
//     tail.
//   * the first call on each device in a process sets up: with the device
//     current it loads this file's device code (the array and both kernels:
//     CUDA loads modules lazily, on first use) and looks up the array's device
//     address (cudaGetSymbolAddress). That first call can allocate device
//     memory; make it, with empty inputs if need be, before a pool reserves
//     the device's memory. Later calls allocate nothing, and the array stays
//     placed until the process exits.
//   * the call is synchronous (it reads the result back before returning), so
//     it must not be made while any stream is being captured.
//   * every call reuses the same array and clears it at the start; calls
//     whose work overlaps on the GPU (different streams, or different host
//     threads without ordering) race on it and must be serialised by the
//     caller.
#include "pg_internal.cuh"
#include <mutex>

#define PG_NOALLOC_SLOTS (1u << 20)                  // 16-byte slots: 16 MiB
#define PG_NOALLOC_LOG2 20
#define PG_NOALLOC_MAX_BUILD (PG_NOALLOC_SLOTS / 2)   // load factor at most 1/2
#define PG_NOALLOC_SIDE 1024                          // build keys equal to the empty marker
#define PG_NOALLOC_WORDS (2u * PG_NOALLOC_SLOTS + PG_NOALLOC_SIDE + 8)

// Layout: [slots: 2 words each][side list][count, sum, side count, flags, ...]
static __device__ __align__(256) unsigned long long g_noalloc_scratch[PG_NOALLOC_WORDS];

struct NaCols {             // packed build value and the summed output column
	int nb;
	uint16_t boff[8];       // word offsets of the build-projected columns
	uint8_t bwords[8];
	int sum_side;           // -1: no sum; 0: build value words; 1: probe tuple
	uint32_t sum_off;       // word offset (packed value, or probe tuple)
	uint32_t sum_words;
};

__device__ __forceinline__ uint64_t na_slot0(int64_t k)
{
	return (pg_mix64((uint64_t) k) >> (65 - PG_NOALLOC_LOG2)) << 1;
}

__global__ void k_na_build(const char* __restrict__ R, uint64_t n, uint32_t W, uint32_t koff,
		uint32_t kbytes, NaCols nc, unsigned long long* __restrict__ scratch)
{
	unsigned long long* slots = scratch;
	unsigned long long* side = scratch + 2ull * PG_NOALLOC_SLOTS;
	unsigned long long* tail = side + PG_NOALLOC_SIDE;
	const uint64_t mask = PG_NOALLOC_SLOTS - 1;
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
			i += (uint64_t) gridDim.x * blockDim.x) {
		const char* t = R + i * W;
		const int64_t k = pg_load_key(t + koff, kbytes);
		uint32_t w[2] = {0, 0};
		int o = 0;
		for (int c = 0; c < nc.nb; ++c)
			for (int j = 0; j < nc.bwords[c]; ++j) w[o++] = reinterpret_cast<const uint32_t*>(t)[nc.boff[c] + j];
		const unsigned long long v = ((unsigned long long) w[1] << 32) | w[0];
		if (k == PG_EMPTY_KEY) {
			const unsigned long long idx = atomicAdd(&tail[2], 1ull);
			if (idx < PG_NOALLOC_SIDE) side[idx] = v; else atomicOr(&tail[3], 2ull);
			continue;
		}
		uint64_t s = na_slot0(k), probe = 0;
		for (; probe <= mask; ++probe) {
			const unsigned long long old = atomicCAS(&slots[2 * s], (unsigned long long) PG_EMPTY_KEY,
					(unsigned long long) k);
			if (old == (unsigned long long) PG_EMPTY_KEY) { slots[2 * s + 1] = v; break; }
			s = (s + 1) & mask;
		}
		if (probe > mask) atomicOr(&tail[3], 1ull);
	}
}

__device__ __forceinline__ unsigned long long na_sum_term(const NaCols& nc, const char* pt, unsigned long long v)
{
	uint32_t lo, hi = 0;
	if (nc.sum_side == 0) {
		lo = nc.sum_off == 0 ? (uint32_t) v : (uint32_t) (v >> 32);
		if (nc.sum_words == 2) hi = (uint32_t) (v >> 32);
	} else {
		lo = reinterpret_cast<const uint32_t*>(pt)[nc.sum_off];
		if (nc.sum_words == 2) hi = reinterpret_cast<const uint32_t*>(pt)[nc.sum_off + 1];
	}
	if (nc.sum_words == 2) return ((unsigned long long) hi << 32) | lo;
	return (unsigned long long) (long long) (int32_t) lo;
}

// Every probe tuple walks its whole probe sequence, so duplicate build keys
// contribute one row each, as in the reference's chain walk (join.cpp:503-562).
__global__ void k_na_probe(const char* __restrict__ S, uint64_t n, uint32_t W, uint32_t koff,
		uint32_t kbytes, NaCols nc, unsigned long long* __restrict__ scratch)
{
	const unsigned long long* slots = scratch;
	const unsigned long long* side = scratch + 2ull * PG_NOALLOC_SLOTS;
	unsigned long long* tail = scratch + 2ull * PG_NOALLOC_SLOTS + PG_NOALLOC_SIDE;
	const uint64_t mask = PG_NOALLOC_SLOTS - 1;
	const unsigned long long nside = tail[2] < PG_NOALLOC_SIDE ? tail[2] : PG_NOALLOC_SIDE;
	unsigned long long cnt = 0, sum = 0;
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
			i += (uint64_t) gridDim.x * blockDim.x) {
		const char* pt = S + i * W;
		const int64_t k = pg_load_key(pt + koff, kbytes);
		if (k == PG_EMPTY_KEY) {
			for (unsigned long long q = 0; q < nside; ++q) {
				++cnt;
				if (nc.sum_side >= 0) sum += na_sum_term(nc, pt, side[q]);
			}
			continue;
		}
		uint64_t s = na_slot0(k);
		for (uint64_t probe = 0; probe <= mask; ++probe) {
			const unsigned long long sk = slots[2 * s];
			if (sk == (unsigned long long) PG_EMPTY_KEY) break;
			if ((long long) sk == k) {
				++cnt;
				if (nc.sum_side >= 0) sum += na_sum_term(nc, pt, slots[2 * s + 1]);
			}
			s = (s + 1) & mask;
		}
	}
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) {
		cnt += __shfl_down_sync(0xffffffffu, cnt, o);
		sum += __shfl_down_sync(0xffffffffu, sum, o);
	}
	if ((threadIdx.x & 31) == 0) { atomicAdd(&tail[0], cnt); atomicAdd(&tail[1], sum); }
}

static std::mutex g_noalloc_mu;
static unsigned long long* g_noalloc_addr[256];

// Makes ctx->device current for one call and restores the caller's device.
struct NaDevice {
	int prev = -1;
	cudaError_t err = cudaSuccess;
	explicit NaDevice(int dev)
	{
		cudaGetDevice(&prev);
		if (prev != dev) err = cudaSetDevice(dev);
	}
	~NaDevice() { if (prev >= 0) cudaSetDevice(prev); }
};

// Device address of g_noalloc_scratch on the current device (ctx->device).
// The first time per device: both kernels are launched once with nothing to
// do, so that their code and the array are loaded now, then the array's
// address is looked up.
static int noalloc_scratch(pg_ctx* ctx, cudaStream_t s, unsigned long long** out)
{
	if (ctx->device < 0 || ctx->device >= 256) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_agg_noalloc: bad device");
	std::lock_guard<std::mutex> g(g_noalloc_mu);
	if (!g_noalloc_addr[ctx->device]) {
		void* p = nullptr;
		cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e != cudaSuccess) return pg_cuda_fail(ctx, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
		unsigned long long* a = static_cast<unsigned long long*>(p);
		NaCols nc = {};
		nc.sum_side = -1;
		k_na_build<<<1, 32, 0, s>>>(nullptr, 0, 16, 0, 8, nc, a);
		k_na_probe<<<1, 32, 0, s>>>(nullptr, 0, 16, 0, 8, nc, a);
		if ((e = cudaGetLastError()) != cudaSuccess) return pg_cuda_fail(ctx, e, "pg_hashjoin_agg_noalloc set-up");
		if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return pg_cuda_fail(ctx, e, "pg_hashjoin_agg_noalloc set-up");
		g_noalloc_addr[ctx->device] = a;
	}
	*out = g_noalloc_addr[ctx->device];
	return PG_OK;
}

extern "C" int pg_hashjoin_agg_noalloc(pg_ctx* ctx, pg_stream stream, const pg_rel* R,
		const pg_rel* S, const pg_col* proj, int nproj, int sum_col, pg_join_result* res)
{
	if (!ctx || !R || !S || !res) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_agg_noalloc: null argument");
	for (const pg_rel* r : {R, S}) {
		if (r->n && !r->data) return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_agg_noalloc: null data");
		if (r->width == 0 || (r->width & 3) || (r->key_bytes != 4 && r->key_bytes != 8) ||
				(r->key_off & 3) || r->key_off + r->key_bytes > r->width)
			return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_agg_noalloc: 4-byte-aligned tuples with an int or long key");
	}
	if (R->n > PG_NOALLOC_MAX_BUILD)
		return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_agg_noalloc: build side above its limit of 524288 tuples");
	if (nproj < 0 || nproj > 8 || (nproj && !proj) || sum_col >= nproj)
		return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_agg_noalloc: 0..8 projected columns, sum_col among them");
	NaCols nc;
	nc.nb = 0; nc.sum_side = -1; nc.sum_off = 0; nc.sum_words = 0;
	uint32_t bwords = 0;
	for (int i = 0; i < nproj; ++i) {
		const pg_col& c = proj[i];
		const uint32_t w = c.side ? S->width : R->width;
		if (c.side > 1 || (c.bytes != 4 && c.bytes != 8) || (c.off & 3) || c.off + c.bytes > w)
			return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_agg_noalloc: projected columns must be 4/8 bytes, aligned");
		if (c.side == 0) {
			if (i == sum_col) { nc.sum_side = 0; nc.sum_off = bwords; nc.sum_words = c.bytes / 4; }
			nc.boff[nc.nb] = (uint16_t) (c.off / 4); nc.bwords[nc.nb] = (uint8_t) (c.bytes / 4); nc.nb++;
			bwords += c.bytes / 4;
		} else if (i == sum_col) {
			nc.sum_side = 1; nc.sum_off = c.off / 4; nc.sum_words = c.bytes / 4;
		}
	}
	if (bwords > 2)
		return pg_fail(ctx, PG_ERR_ARG, "pg_hashjoin_agg_noalloc: build-side columns limited to 8 bytes in total");
	NaDevice dev(ctx->device);
	if (dev.err != cudaSuccess) return pg_cuda_fail(ctx, dev.err, "pg_hashjoin_agg_noalloc: cudaSetDevice");
	cudaStream_t s = (cudaStream_t) stream;
	unsigned long long* scratch = nullptr;
	int rc;
	if ((rc = noalloc_scratch(ctx, s, &scratch))) return rc;
	unsigned long long* tail = scratch + 2ull * PG_NOALLOC_SLOTS + PG_NOALLOC_SIDE;
	// The array keeps the previous call's contents: clear the table and the tail.
	PG_CUDA(ctx, cudaMemsetAsync(scratch, 0xFF, 2ull * PG_NOALLOC_SLOTS * 8, s));
	PG_CUDA(ctx, cudaMemsetAsync(tail, 0, 8 * 8, s));
	const int bb = (int) std::min<uint64_t>(pg_div_up(std::max<uint64_t>(R->n, 1), 256), (uint64_t) ctx->sm_count * 8);
	if (R->n) {
		k_na_build<<<bb, 256, 0, s>>>((const char*) R->data, R->n, R->width, R->key_off, R->key_bytes, nc, scratch);
		PG_LAUNCHED(ctx);
	}
	const int pb = (int) std::min<uint64_t>(pg_div_up(std::max<uint64_t>(S->n, 1), 256), (uint64_t) ctx->sm_count * 16);
	if (S->n && R->n) {
		k_na_probe<<<pb, 256, 0, s>>>((const char*) S->data, S->n, S->width, S->key_off, S->key_bytes, nc, scratch);
		PG_LAUNCHED(ctx);
	}
	unsigned long long h[4] = {0, 0, 0, 0};
	PG_CUDA(ctx, cudaMemcpyAsync(h, tail, sizeof h, cudaMemcpyDeviceToHost, s));
	PG_CUDA(ctx, cudaStreamSynchronize(s));
	if (h[3] & 2) return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_hashjoin_agg_noalloc: more than 1024 build keys equal -1");
	if (h[3] & 1) return pg_fail(ctx, PG_ERR_TABLE_FULL, "pg_hashjoin_agg_noalloc: table full");
	res->n_out = h[0];
	res->sum = sum_col >= 0 ? (int64_t) h[1] : 0;
	return PG_OK;
}
