// Context, memory, error plumbing, tuple hashing and the device scan used by
// every operator of libpythia_gpu.
#include "pg_internal.cuh"
#include <cstring>
#include <algorithm>
#include <cstdio>

std::atomic<uint64_t> g_kernel_launches{0};

static thread_local std::string t_last_error;

int pg_fail(pg_ctx* ctx, int code, const std::string& msg)
{
	t_last_error = msg;
	if (ctx) {
		std::lock_guard<std::mutex> g(ctx->mu);
		ctx->last_error = msg;
	}
	return code;
}

int pg_cuda_fail(pg_ctx* ctx, cudaError_t e, const char* what)
{
	std::string m = std::string(what) + ": " + cudaGetErrorString(e);
	return pg_fail(ctx, e == cudaErrorMemoryAllocation ? PG_ERR_OOM : PG_ERR_CUDA, m);
}

extern "C" uint64_t pg_kernel_launches(void) { return g_kernel_launches.load(); }

extern "C" int pg_tune_set(pg_ctx* ctx, int knob, int64_t value)
{
	if (!ctx || knob < 0 || knob >= PG_TUNE_COUNT || value < 0)
		return pg_fail(ctx, PG_ERR_ARG, "pg_tune_set: unknown knob or negative value");
	ctx->tune[knob] = value;
	if (knob == PG_TUNE_SPIN_LIMIT) {
		// Kernels read the limit from word 1 of the device status block.
		const uint32_t v = (uint32_t) std::min<int64_t>(value, (int64_t) PG_SPIN_LIMIT);
		PG_CUDA(ctx, cudaMemcpy(ctx->d_status + 1, &v, sizeof v, cudaMemcpyHostToDevice));
	}
	if (knob == PG_TUNE_L2_FETCH && value) {
		// A hint of how many bytes an L2 miss fetches from DRAM; random 32-byte
		// bucket reads of a table larger than L2 want the smallest.
		if (value != 32 && value != 64 && value != 128)
			return pg_fail(ctx, PG_ERR_ARG, "pg_tune_set: L2 fetch granularity must be 32, 64 or 128");
		PG_CUDA(ctx, cudaSetDevice(ctx->device));
		PG_CUDA(ctx, cudaDeviceSetLimit(cudaLimitMaxL2FetchGranularity, (size_t) value));
	}
	return PG_OK;
}

extern "C" int64_t pg_tune_get(pg_ctx* ctx, int knob)
{
	if (!ctx || knob < 0 || knob >= PG_TUNE_COUNT) return -1;
	return ctx->tune[knob];
}

extern "C" int pg_init(int device, uint64_t reserved_bytes, pg_ctx** out)
{
	if (!out) return pg_fail(nullptr, PG_ERR_ARG, "pg_init: null ctx pointer");
	int ndev = 0;
	cudaError_t e = cudaGetDeviceCount(&ndev);
	if (e != cudaSuccess || ndev == 0)
		return pg_fail(nullptr, PG_ERR_CUDA, "pg_init: no CUDA device available");
	if (device < 0 || device >= ndev) return pg_fail(nullptr, PG_ERR_ARG, "pg_init: bad device");
	pg_ctx* ctx = new pg_ctx();
	ctx->device = device;
	for (int i = 0; i < PG_TUNE_COUNT; ++i) ctx->tune[i] = 0;
	if ((e = cudaSetDevice(device)) != cudaSuccess) { delete ctx; return pg_cuda_fail(nullptr, e, "cudaSetDevice"); }
	cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, device);
	ctx->pageable_access = 0;
	ctx->host_ptr_registered = 0;
	cudaDeviceGetAttribute(&ctx->pageable_access, cudaDevAttrPageableMemoryAccess, device);
	cudaDeviceGetAttribute(&ctx->host_ptr_registered, cudaDevAttrCanUseHostPointerForRegisteredMem, device);
	cudaDeviceGetDefaultMemPool(&ctx->pool, device);
	// Keep freed blocks in the pool: operators allocate scratch per call.
	uint64_t thresh = UINT64_MAX;
	cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &thresh);
	// Large buffers (join outputs, gathered inputs) come from a pool of their
	// own: interleaved with the many smaller staging chunks they left the
	// shared pool too fragmented to reuse, and a 1 GB output then mapped new
	// memory on every plan run (about 1.1 ms).
	ctx->big_pool = nullptr;
	cudaMemPoolProps props;
	memset(&props, 0, sizeof(props));
	props.allocType = cudaMemAllocationTypePinned;
	props.location.type = cudaMemLocationTypeDevice;
	props.location.id = device;
	if (cudaMemPoolCreate(&ctx->big_pool, &props) == cudaSuccess)
		cudaMemPoolSetAttribute(ctx->big_pool, cudaMemPoolAttrReleaseThreshold, &thresh);
	else { ctx->big_pool = nullptr; cudaGetLastError(); }
	if (reserved_bytes) {
		// Warm the pool so the first operator does not pay for growth.
		void* p = nullptr;
		if (cudaMallocAsync(&p, reserved_bytes, 0) == cudaSuccess) cudaFreeAsync(p, 0);
		cudaStreamSynchronize(0);
		cudaGetLastError();
	}
	if ((e = cudaMalloc(&ctx->d_status, 4096)) != cudaSuccess) { delete ctx; return pg_cuda_fail(nullptr, e, "cudaMalloc status"); }
	cudaMemset(ctx->d_status, 0, 4096);
	ctx->d_scratch64 = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(ctx->d_status) + 256);
	cudaDeviceSynchronize();
	*out = ctx;
	return PG_OK;
}

extern "C" int pg_shutdown(pg_ctx* ctx)
{
	if (!ctx) return PG_ERR_ARG;
	cudaSetDevice(ctx->device);
	cudaDeviceSynchronize();
	cudaFree(ctx->d_status);
	// Released once its last allocation is freed, if any is still out.
	if (ctx->big_pool) cudaMemPoolDestroy(ctx->big_pool);
	delete ctx;
	return PG_OK;
}

extern "C" const char* pg_last_error(pg_ctx* ctx)
{
	(void) ctx;
	return t_last_error.c_str();
}

extern "C" int pg_device_status(pg_ctx* ctx)
{
	if (!ctx) return PG_ERR_ARG;
	int st = 0;
	PG_CUDA(ctx, cudaMemcpy(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost));
	return st;
}

int pg_status_fail(pg_ctx* ctx, cudaStream_t s, int st, const char* what)
{
	cudaMemsetAsync(ctx->d_status, 0, sizeof(int), s);
	cudaStreamSynchronize(s);
	const char* why = st == PG_ERR_TIMEOUT ? "a bounded device wait gave up"
		: st == PG_ERR_TABLE_FULL ? "hash table probe sequence exhausted" : "device error";
	return pg_fail(ctx, st, std::string(what) + ": " + why);
}

int pg_check_status(pg_ctx* ctx, cudaStream_t s, const char* what)
{
	// Stream-ordered read of the status word: no synchronisation with other
	// streams, one round trip for the wait and the read.
	int st = 0;
	PG_CUDA(ctx, cudaMemcpyAsync(&st, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
	PG_CUDA(ctx, cudaStreamSynchronize(s));
	if (st) return pg_status_fail(ctx, s, st, what);
	return PG_OK;
}

extern "C" int pg_stream_create(pg_ctx* ctx, pg_stream* s)
{
	if (!ctx || !s) return PG_ERR_ARG;
	cudaStream_t st;
	PG_CUDA(ctx, cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
	*s = st;
	return PG_OK;
}

extern "C" int pg_stream_create_urgent(pg_ctx* ctx, pg_stream* s)
{
	if (!ctx || !s) return PG_ERR_ARG;
	int least = 0, greatest = 0;
	PG_CUDA(ctx, cudaDeviceGetStreamPriorityRange(&least, &greatest));
	cudaStream_t st;
	PG_CUDA(ctx, cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, greatest));
	*s = st;
	return PG_OK;
}

extern "C" int pg_stream_destroy(pg_ctx* ctx, pg_stream s)
{
	if (!ctx) return PG_ERR_ARG;
	PG_CUDA(ctx, cudaStreamDestroy((cudaStream_t) s));
	return PG_OK;
}

extern "C" int pg_sync(pg_ctx* ctx, pg_stream s)
{
	if (!ctx) return PG_ERR_ARG;
	PG_CUDA(ctx, cudaStreamSynchronize((cudaStream_t) s));
	return PG_OK;
}

extern "C" int pg_buffer_alloc(pg_ctx* ctx, uint64_t bytes, void** p)
{
	if (!ctx || !p) return PG_ERR_ARG;
	PG_CUDA(ctx, cudaMalloc(p, bytes ? bytes : 16));
	return PG_OK;
}

extern "C" int pg_buffer_free(pg_ctx* ctx, void* p)
{
	if (!ctx) return PG_ERR_ARG;
	PG_CUDA(ctx, cudaFree(p));
	return PG_OK;
}

extern "C" int pg_buffer_alloc_async(pg_ctx* ctx, pg_stream s, uint64_t bytes, void** p)
{
	if (!ctx || !p) return PG_ERR_ARG;
	return pg_alloc_async(ctx, (cudaStream_t) s, p, bytes);
}

extern "C" int pg_buffer_free_async(pg_ctx* ctx, pg_stream s, void* p)
{
	if (!ctx) return PG_ERR_ARG;
	pg_free_async(ctx, (cudaStream_t) s, p);
	return PG_OK;
}

extern "C" int pg_host_alloc(pg_ctx* ctx, uint64_t bytes, void** p)
{
	if (!ctx || !p) return PG_ERR_ARG;
	PG_CUDA(ctx, cudaMallocHost(p, bytes ? bytes : 16));
	return PG_OK;
}

extern "C" int pg_host_register(pg_ctx* ctx, void* p, uint64_t bytes)
{
	if (!ctx || (!p && bytes)) return pg_fail(ctx, PG_ERR_ARG, "pg_host_register: null argument");
	if (bytes) PG_CUDA(ctx, cudaHostRegister(p, bytes, cudaHostRegisterDefault));
	return PG_OK;
}

extern "C" int pg_host_unregister(pg_ctx* ctx, void* p)
{
	if (!ctx) return PG_ERR_ARG;
	if (p) PG_CUDA(ctx, cudaHostUnregister(p));
	return PG_OK;
}

extern "C" int pg_host_is_pinned(pg_ctx* ctx, const void* p)
{
	if (!ctx || !p) return 0;
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) { cudaGetLastError(); return 0; }
	return a.type == cudaMemoryTypeHost ? 1 : 0;
}

extern "C" int pg_host_readable(pg_ctx* ctx, const void* p)
{
	if (!ctx || !p) return 0;
	return pg_host_is_pinned(ctx, p) || ctx->pageable_access ? 1 : 0;
}

// Host-to-device copy by the SMs: bytes [0, head) one per thread until dst is
// 16-byte aligned, then units of U (the widest that src + head allows), then
// the remaining bytes one per thread.
template <typename U>
__global__ void k_sm_copy(const char* __restrict__ src, char* __restrict__ dst, uint64_t n, uint32_t head)
{
	const uint64_t tid = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x;
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	if (tid < head) dst[tid] = src[tid];
	const uint64_t units = (n - head) / sizeof(U);
	const U* s = reinterpret_cast<const U*>(src + head);
	U* d = reinterpret_cast<U*>(dst + head);
	for (uint64_t i = tid; i < units; i += stride) d[i] = s[i];
	const uint64_t done = head + units * sizeof(U);
	if (tid < n - done) dst[done + tid] = src[done + tid];
}

extern "C" int pg_h2d_sm(pg_ctx* ctx, pg_stream stream, void* dst, const void* src, uint64_t bytes)
{
	if (!ctx) return PG_ERR_ARG;
	if (!bytes) return PG_OK;
	if (!dst || !src) return pg_fail(ctx, PG_ERR_ARG, "pg_h2d_sm: null pointer");
	const char* from = (const char*) src;
	if (pg_host_is_pinned(ctx, src)) {
		if (!ctx->host_ptr_registered) {
			void* d = nullptr;
			PG_CUDA(ctx, cudaHostGetDevicePointer(&d, const_cast<void*>(src), 0));
			from = (const char*) d;
		}
	} else if (!ctx->pageable_access) {
		return pg_fail(ctx, PG_ERR_ARG, "pg_h2d_sm: host memory the device cannot read (not pinned, no pageable access)");
	}
	cudaStream_t s = (cudaStream_t) stream;
	const uint32_t head = (uint32_t) std::min<uint64_t>(bytes, (16 - (reinterpret_cast<uintptr_t>(dst) & 15)) & 15);
	const uintptr_t a = reinterpret_cast<uintptr_t>(from + head);
	const uint32_t unit = (a & 15) == 0 ? 16 : (a & 7) == 0 ? 8 : (a & 3) == 0 ? 4 : 1;
	const uint64_t units = (bytes - head) / unit;
	const int blocks = (int) std::max<uint64_t>(1, std::min<uint64_t>(pg_div_up(units, 256 * 4), (uint64_t) ctx->sm_count * 2));
	char* to = (char*) dst;
	if (unit == 16) k_sm_copy<uint4><<<blocks, 256, 0, s>>>(from, to, bytes, head);
	else if (unit == 8) k_sm_copy<uint2><<<blocks, 256, 0, s>>>(from, to, bytes, head);
	else if (unit == 4) k_sm_copy<uint32_t><<<blocks, 256, 0, s>>>(from, to, bytes, head);
	else k_sm_copy<unsigned char><<<blocks, 256, 0, s>>>(from, to, bytes, head);
	PG_LAUNCHED(ctx);
	return PG_OK;
}

extern "C" int pg_host_free(pg_ctx* ctx, void* p)
{
	if (!ctx) return PG_ERR_ARG;
	PG_CUDA(ctx, cudaFreeHost(p));
	return PG_OK;
}

extern "C" int pg_h2d(pg_ctx* ctx, pg_stream s, void* dst, const void* src, uint64_t bytes)
{
	if (!ctx) return PG_ERR_ARG;
	if (bytes) PG_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t) s));
	return PG_OK;
}

extern "C" int pg_d2h(pg_ctx* ctx, pg_stream s, void* dst, const void* src, uint64_t bytes)
{
	if (!ctx) return PG_ERR_ARG;
	if (bytes) PG_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t) s));
	return PG_OK;
}

extern "C" int pg_d2d(pg_ctx* ctx, pg_stream s, void* dst, const void* src, uint64_t bytes)
{
	if (!ctx) return PG_ERR_ARG;
	if (bytes) PG_CUDA(ctx, cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t) s));
	return PG_OK;
}

extern "C" int pg_memset(pg_ctx* ctx, pg_stream s, void* dst, int value, uint64_t bytes)
{
	if (!ctx) return PG_ERR_ARG;
	if (bytes) PG_CUDA(ctx, cudaMemsetAsync(dst, value, bytes, (cudaStream_t) s));
	return PG_OK;
}

int pg_alloc_async(pg_ctx* ctx, cudaStream_t s, void** p, size_t bytes)
{
	cudaMemPool_t pool = bytes >= PG_BIG_ALLOC && ctx->big_pool ? ctx->big_pool : ctx->pool;
	cudaError_t e = cudaMallocFromPoolAsync(p, bytes ? bytes : 16, pool, s);
	if (e != cudaSuccess) return pg_cuda_fail(ctx, e, "cudaMallocFromPoolAsync");
	return PG_OK;
}

void pg_free_async(pg_ctx* ctx, cudaStream_t s, void* p)
{
	(void) ctx;
	if (p) cudaFreeAsync(p, s);
}

// ---------------------------------------------------------------------------
// Bucket functions: the constructors of hash.h:51-479 as TupleHasher::create
// (hash.cpp:99-215) calls them, and getlogarithm (hash.cpp:47-56).
// ---------------------------------------------------------------------------
static uint32_t getlogarithm(uint32_t k)
{
	--k;
	for (uint32_t i = 0; i < 32; ++i)
		if ((0x80000000u >> i) & k) return 32 - i;
	return 0;
}

int pg_hashfn_derive(const pg_hashcfg* c, pg_hashfn* f)
{
	memset(f, 0, sizeof *f);
	f->fn = c->fn;
	switch (c->fn) {
	case PG_FN_ALWAYSZERO: f->nbuckets = 1; return PG_OK;
	case PG_FN_TPCHQ1MAGIC: f->k = 2; f->nbuckets = 4; return PG_OK;
	default: break;
	}
	if (c->buckets == 0) return PG_ERR_ARG;
	uint32_t lg = getlogarithm(c->buckets);
	switch (c->fn) {
	case PG_FN_BYTES: f->k = lg; f->nbuckets = 1u << lg; break;
	case PG_FN_MODULO: case PG_FN_TPCHORDERKEY: case PG_FN_WILLIS:
		f->k = (int64_t) ((1 << lg) - 1); f->nbuckets = (uint32_t) f->k + 1; break;
	case PG_FN_RANGE:
		f->k = lg; f->min = c->min; f->max = c->max; f->nbuckets = 1u << lg; break;
	case PG_FN_EXACTRANGE:
		f->min = c->min; f->max = c->max; f->k = c->buckets;
		f->bucketrange = (f->max - f->min + f->k) / f->k;
		if (f->bucketrange <= 0) return PG_ERR_ARG;
		f->nbuckets = c->buckets; break;
	case PG_FN_PARAMMODULO: case PG_FN_KNUTH:
		f->k = (int64_t) ((1 << lg) - 1);
		f->skipbits = c->skipbits;
		f->k <<= c->skipbits;
		f->min = (int64_t) c->offset;
		f->nbuckets = (uint32_t) (f->k >> f->skipbits) + 1;
		break;
	default: return PG_ERR_ARG;
	}
	return PG_OK;
}

extern "C" int pg_hash_buckets(pg_ctx* ctx, const pg_hashcfg* cfg, uint32_t* nb)
{
	if (!cfg || !nb) return pg_fail(ctx, PG_ERR_ARG, "pg_hash_buckets: null argument");
	pg_hashfn f;
	if (pg_hashfn_derive(cfg, &f)) return pg_fail(ctx, PG_ERR_ARG, "pg_hash_buckets: invalid hash configuration");
	*nb = f.nbuckets;
	return PG_OK;
}

__global__ void k_hash_tuples(const char* __restrict__ in, uint64_t n, uint32_t width,
		uint32_t koff, uint32_t kbytes, pg_hashfn f, uint32_t* __restrict__ out)
{
	for (uint64_t i = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; i < n;
			i += (uint64_t) gridDim.x * blockDim.x)
		out[i] = pg_hash_field(f, in + i * width + koff, kbytes);
}

extern "C" int pg_hash_tuples(pg_ctx* ctx, pg_stream stream, const pg_rel* in,
		const pg_hashcfg* cfg, uint32_t* out)
{
	if (!ctx || !in || !cfg) return pg_fail(ctx, PG_ERR_ARG, "pg_hash_tuples: null argument");
	pg_hashfn f;
	if (pg_hashfn_derive(cfg, &f)) return pg_fail(ctx, PG_ERR_ARG, "pg_hash_tuples: invalid hash configuration");
	if (in->n == 0) return PG_OK;
	if (in->key_off + in->key_bytes > in->width) return pg_fail(ctx, PG_ERR_ARG, "pg_hash_tuples: key outside tuple");
	int blocks = (int) std::min<uint64_t>(pg_div_up(in->n, 256), (uint64_t) ctx->sm_count * 16);
	k_hash_tuples<<<blocks, 256, 0, (cudaStream_t) stream>>>((const char*) in->data, in->n,
			in->width, in->key_off, in->key_bytes, f, out);
	PG_LAUNCHED(ctx);
	return PG_OK;
}

// ---------------------------------------------------------------------------
// Exclusive scan of uint64 values (three phases: block sums, recursive scan
// of the sums, block-local scan plus offset).
// ---------------------------------------------------------------------------
#define SCAN_THREADS 256
#define SCAN_ITEMS 8
#define SCAN_TILE (SCAN_THREADS * SCAN_ITEMS)

__device__ __forceinline__ uint64_t block_excl_scan(uint64_t v, uint64_t* warp_tot, uint64_t* total)
{
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	uint64_t x = v;
	#pragma unroll
	for (int o = 1; o < 32; o <<= 1) {
		uint64_t y = __shfl_up_sync(0xffffffffu, x, o);
		if (lane >= o) x += y;
	}
	if (lane == 31) warp_tot[warp] = x;
	__syncthreads();
	if (warp == 0) {
		uint64_t t = lane < (SCAN_THREADS / 32) ? warp_tot[lane] : 0;
		uint64_t tt = t;
		#pragma unroll
		for (int o = 1; o < 32; o <<= 1) {
			uint64_t y = __shfl_up_sync(0xffffffffu, tt, o);
			if (lane >= o) tt += y;
		}
		if (lane < (SCAN_THREADS / 32)) warp_tot[lane] = tt - t;
		if (lane == (SCAN_THREADS / 32) - 1) *total = tt;
	}
	__syncthreads();
	uint64_t r = x - v + warp_tot[warp];
	__syncthreads();
	return r;
}

__global__ void k_scan_sums(const uint64_t* __restrict__ d, uint64_t n, uint64_t* __restrict__ sums)
{
	__shared__ uint64_t wt[SCAN_THREADS / 32];
	__shared__ uint64_t tot;
	uint64_t base = (uint64_t) blockIdx.x * SCAN_TILE + (uint64_t) threadIdx.x * SCAN_ITEMS;
	uint64_t s = 0;
	#pragma unroll
	for (int j = 0; j < SCAN_ITEMS; ++j) if (base + j < n) s += d[base + j];
	block_excl_scan(s, wt, &tot);
	if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void k_scan_apply(uint64_t* __restrict__ d, uint64_t n, const uint64_t* __restrict__ offs)
{
	__shared__ uint64_t wt[SCAN_THREADS / 32];
	__shared__ uint64_t tot;
	uint64_t base = (uint64_t) blockIdx.x * SCAN_TILE + (uint64_t) threadIdx.x * SCAN_ITEMS;
	uint64_t v[SCAN_ITEMS], s = 0;
	#pragma unroll
	for (int j = 0; j < SCAN_ITEMS; ++j) { v[j] = base + j < n ? d[base + j] : 0; s += v[j]; }
	uint64_t run = block_excl_scan(s, wt, &tot) + (offs ? offs[blockIdx.x] : 0);
	#pragma unroll
	for (int j = 0; j < SCAN_ITEMS; ++j) {
		if (base + j < n) d[base + j] = run;
		run += v[j];
	}
}

__global__ void k_scan_total(const uint64_t* __restrict__ d, const uint64_t* __restrict__ last_in,
		uint64_t n, uint64_t* __restrict__ total)
{
	*total = n ? d[n - 1] + *last_in : 0;
}

int pg_scan_u64(pg_ctx* ctx, cudaStream_t s, uint64_t* data, uint64_t n, uint64_t* total_dev)
{
	if (n == 0) {
		if (total_dev) PG_CUDA(ctx, cudaMemsetAsync(total_dev, 0, 8, s));
		return PG_OK;
	}
	uint64_t nb = pg_div_up(n, SCAN_TILE);
	uint64_t* last = nullptr;
	int rc;
	if (total_dev) {
		if ((rc = pg_alloc_async(ctx, s, (void**) &last, 8))) return rc;
		PG_CUDA(ctx, cudaMemcpyAsync(last, data + n - 1, 8, cudaMemcpyDeviceToDevice, s));
	}
	if (nb == 1) {
		k_scan_apply<<<1, SCAN_THREADS, 0, s>>>(data, n, nullptr);
		PG_LAUNCHED(ctx);
	} else {
		uint64_t* sums = nullptr;
		if ((rc = pg_alloc_async(ctx, s, (void**) &sums, nb * 8))) return rc;
		k_scan_sums<<<(unsigned) nb, SCAN_THREADS, 0, s>>>(data, n, sums);
		PG_LAUNCHED(ctx);
		if ((rc = pg_scan_u64(ctx, s, sums, nb, nullptr))) return rc;
		k_scan_apply<<<(unsigned) nb, SCAN_THREADS, 0, s>>>(data, n, sums);
		PG_LAUNCHED(ctx);
		pg_free_async(ctx, s, sums);
	}
	if (total_dev) {
		k_scan_total<<<1, 1, 0, s>>>(data, last, n, total_dev);
		PG_LAUNCHED(ctx);
		pg_free_async(ctx, s, last);
	}
	return PG_OK;
}
