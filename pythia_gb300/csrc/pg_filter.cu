// Filter and Project on sm_103a.
//
// Replace Filter::map and Project::map (operators/filter.cpp:37-85,
// project.cpp:37-104), which MapWrapper calls tuple by tuple per thread
// (mapwrapper.cpp:38-138), with one launch over the whole relation.
//
// Filter is a stable compaction in two passes over tiles of 2048 tuples: the
// first evaluates the predicates and counts survivors per tile, an exclusive
// scan turns counts into output offsets, and the second re-evaluates and
// writes each survivor at its tile offset plus its rank in input order (warp
// ballots, then warp totals in shared memory). Both passes stream the input
// once, so the traffic is two reads of the relation and one write of the
// survivors. Project stages tiles in shared memory so that both its loads and
// its stores are coalesced: one read, one write.
#include "pg_pred.cuh"
#include <algorithm>
#include <cstring>

#define FL_THREADS 256
#define FL_ITEMS 8
#define FL_TILE (FL_THREADS * FL_ITEMS)
#define HJ_PROJ_MAX 16

int pg_pred_prepare(pg_ctx* ctx, const pg_pred* preds, int npred, uint32_t width, PgPredSet* out, bool* has_char)
{
	if (npred < 0 || npred > PG_PRED_MAX || (npred && !preds))
		return pg_fail(ctx, PG_ERR_ARG, "predicates: 0..4 predicates");
	memset(out, 0, sizeof(*out));
	out->n = npred;
	*has_char = false;
	for (int i = 0; i < npred; ++i) {
		const pg_pred& p = preds[i];
		if (p.op > PG_CMP_GE) return pg_fail(ctx, PG_ERR_ARG, "predicates: unknown comparison");
		const bool num = p.type == PG_PRED_INT || p.type == PG_PRED_LONG || p.type == PG_PRED_DEC;
		if (num) {
			const uint32_t want = p.type == PG_PRED_INT ? 4 : 8;
			if (p.bytes != want || (p.off & 3) || p.off + p.bytes > width)
				return pg_fail(ctx, PG_ERR_ARG, "predicates: int 4 bytes, long/dec 8 bytes, 4-byte aligned, inside the tuple");
			uint64_t v = 0;
			memcpy(&v, p.value, p.bytes);
			out->v[i] = v;
		} else if (p.type == PG_PRED_CHAR) {
			if (p.bytes < 1 || p.bytes > 128 || p.off + p.bytes > width)
				return pg_fail(ctx, PG_ERR_ARG, "predicates: char columns of 1..128 bytes inside the tuple");
			*has_char = true;
		} else {
			return pg_fail(ctx, PG_ERR_ARG, "predicates: unknown column type");
		}
		out->type[i] = p.type; out->op[i] = p.op; out->off[i] = p.off; out->bytes[i] = p.bytes;
	}
	return PG_OK;
}

bool pg_pred_as16(const pg_pred* preds, int npred, PgPred16* out)
{
	memset(out, 0, sizeof(*out));
	out->n = npred;
	for (int i = 0; i < npred; ++i) {
		const pg_pred& p = preds[i];
		if (p.type == PG_PRED_CHAR || (p.off & 3) || p.off + p.bytes > 16) return false;
		out->word[i] = (uint8_t) (p.off / 4);
		out->type[i] = (uint8_t) p.type;
		out->op[i] = (uint8_t) p.op;
		uint64_t v = 0;
		memcpy(&v, p.value, p.type == PG_PRED_INT ? 4 : 8);
		out->v[i] = v;
	}
	return true;
}

// Survivors per tile of FL_TILE tuples (index order j * 256 + thread).
__global__ void __launch_bounds__(FL_THREADS)
k_filter_count(const char* __restrict__ in, uint64_t n, uint32_t w, const PgPredSet P, uint64_t* __restrict__ counts)
{
	__shared__ uint32_t wsum[FL_THREADS / 32];
	const uint64_t base = (uint64_t) blockIdx.x * FL_TILE;
	uint32_t c = 0;
	#pragma unroll
	for (int j = 0; j < FL_ITEMS; ++j) {
		const uint64_t i = base + j * FL_THREADS + threadIdx.x;
		if (i < n && pg_pred_eval(P, in + i * w)) ++c;
	}
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
	if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = c;
	__syncthreads();
	if (threadIdx.x == 0) {
		uint32_t t = 0;
		for (int k = 0; k < FL_THREADS / 32; ++k) t += wsum[k];
		counts[blockIdx.x] = t;
	}
}

// 16-byte tuples and numeric predicates: whole-tuple vector loads and the
// predicates evaluated on the registers.
__global__ void __launch_bounds__(FL_THREADS)
k_filter_count16(const uint4* __restrict__ in, uint64_t n, const PgPred16 P, uint64_t* __restrict__ counts)
{
	__shared__ uint32_t wsum[FL_THREADS / 32];
	const uint64_t base = (uint64_t) blockIdx.x * FL_TILE;
	uint4 t[FL_ITEMS];
	#pragma unroll
	for (int j = 0; j < FL_ITEMS; ++j) {
		const uint64_t i = base + j * FL_THREADS + threadIdx.x;
		t[j] = i < n ? __ldcs(in + i) : make_uint4(0, 0, 0, 0);
	}
	uint32_t c = 0;
	#pragma unroll
	for (int j = 0; j < FL_ITEMS; ++j) {
		const uint64_t i = base + j * FL_THREADS + threadIdx.x;
		if (i < n && pg_pred16(P, t[j])) ++c;
	}
	#pragma unroll
	for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
	if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = c;
	__syncthreads();
	if (threadIdx.x == 0) {
		uint32_t tot = 0;
		for (int k = 0; k < FL_THREADS / 32; ++k) tot += wsum[k];
		counts[blockIdx.x] = tot;
	}
}

// vec: tuples start on 16-byte boundaries (width and both bases multiples of 16).
__device__ __forceinline__ void fl_copy(char* __restrict__ dst, const char* __restrict__ src, uint32_t w, bool vec)
{
	if (vec) {
		for (uint32_t b = 0; b < w; b += 16)
			*reinterpret_cast<uint4*>(dst + b) = __ldcs(reinterpret_cast<const uint4*>(src + b));
	} else {
		for (uint32_t b = 0; b < w; b += 4)
			*reinterpret_cast<uint32_t*>(dst + b) = __ldcs(reinterpret_cast<const uint32_t*>(src + b));
	}
}

// Writes each tile's survivors at offs[tile] in input order. All of a
// thread's items are loaded (16-byte tuples into registers) and evaluated
// before the block ranks them, so eight loads per thread are in flight and
// the tile needs two barriers.
// REG16 (with VEC16): the predicates are evaluated on the loaded registers.
template <bool VEC16, bool REG16>
__global__ void __launch_bounds__(FL_THREADS, 4)
k_filter_write(const char* __restrict__ in, uint64_t n, uint32_t w, const PgPredSet P, const PgPred16 P16,
		const uint64_t* __restrict__ offs, char* __restrict__ out, bool vec)
{
	__shared__ uint32_t cnt[FL_ITEMS][FL_THREADS / 32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
	const uint64_t base = (uint64_t) blockIdx.x * FL_TILE;
	uint4 t[VEC16 ? FL_ITEMS : 1];
	if (VEC16) {
		#pragma unroll
		for (int j = 0; j < FL_ITEMS; ++j) {
			const uint64_t i = base + j * FL_THREADS + threadIdx.x;
			t[VEC16 ? j : 0] = i < n ? __ldcs(reinterpret_cast<const uint4*>(in) + i) : make_uint4(0, 0, 0, 0);
		}
	}
	uint32_t ball[FL_ITEMS];
	#pragma unroll
	for (int j = 0; j < FL_ITEMS; ++j) {
		const uint64_t i = base + j * FL_THREADS + threadIdx.x;
		ball[j] = __ballot_sync(0xffffffffu, i < n && (REG16 ? pg_pred16(P16, t[VEC16 ? j : 0])
				: pg_pred_eval(P, in + i * w)));
		if (lane == 0) cnt[j][warp] = __popc(ball[j]);
	}
	__syncthreads();
	if (threadIdx.x == 0) {
		uint32_t run = 0;
		for (int j = 0; j < FL_ITEMS; ++j)
			for (int k = 0; k < FL_THREADS / 32; ++k) { const uint32_t c = cnt[j][k]; cnt[j][k] = run; run += c; }
	}
	__syncthreads();
	const uint64_t at = offs[blockIdx.x];
	#pragma unroll
	for (int j = 0; j < FL_ITEMS; ++j) {
		if (!((ball[j] >> lane) & 1)) continue;
		const uint64_t i = base + j * FL_THREADS + threadIdx.x;
		const uint64_t o = at + cnt[j][warp] + __popc(ball[j] & ((1u << lane) - 1));
		if (VEC16) __stcs(reinterpret_cast<uint4*>(out) + o, t[VEC16 ? j : 0]);
		else fl_copy(out + o * w, in + i * w, w, vec);
	}
}

extern "C" int pg_filter(pg_ctx* ctx, pg_stream stream, const pg_rel* in, const pg_pred* preds, int npred,
		void* out, uint64_t* n_out)
{
	if (!ctx || !in || !n_out) return pg_fail(ctx, PG_ERR_ARG, "pg_filter: null argument");
	if (in->n && (!in->data || !out)) return pg_fail(ctx, PG_ERR_ARG, "pg_filter: null data");
	if (in->width == 0 || (in->width & 3)) return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_filter: tuple width must be a multiple of 4");
	if (in->n && ((reinterpret_cast<uintptr_t>(in->data) | reinterpret_cast<uintptr_t>(out)) & 3))
		return pg_fail(ctx, PG_ERR_ARG, "pg_filter: data must be 4-byte aligned");
	PgPredSet P;
	bool has_char = false;
	int rc;
	if ((rc = pg_pred_prepare(ctx, preds, npred, in->width, &P, &has_char))) return rc;
	*n_out = 0;
	if (in->n == 0) return PG_OK;
	cudaStream_t s = (cudaStream_t) stream;
	const bool vec = (in->width & 15) == 0 && ((reinterpret_cast<uintptr_t>(in->data) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
	const uint32_t w = in->width;
	const uint64_t ntiles = pg_div_up(in->n, FL_TILE);
	uint64_t* offs = nullptr;
	uint8_t* chars = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &offs, (ntiles + 1) * 8))) return rc;
	if (has_char) {
		uint8_t host[PG_PRED_MAX * 128];
		memset(host, 0, sizeof host);
		for (int i = 0; i < npred; ++i) memcpy(host + i * 128, preds[i].value, 128);
		if ((rc = pg_alloc_async(ctx, s, (void**) &chars, sizeof host))) return rc;
		PG_CUDA(ctx, cudaMemcpyAsync(chars, host, sizeof host, cudaMemcpyHostToDevice, s));
		PG_CUDA(ctx, cudaStreamSynchronize(s));     // `host` leaves scope
		P.chars = chars;
	}
	PgPred16 P16;
	const bool reg16 = vec && w == 16 && pg_pred_as16(preds, npred, &P16);
	if (reg16)
		k_filter_count16<<<(unsigned) ntiles, FL_THREADS, 0, s>>>((const uint4*) in->data, in->n, P16, offs);
	else
		k_filter_count<<<(unsigned) ntiles, FL_THREADS, 0, s>>>((const char*) in->data, in->n, w, P, offs);
	PG_LAUNCHED(ctx);
	if ((rc = pg_scan_u64(ctx, s, offs, ntiles, offs + ntiles))) return rc;
	if (reg16)
		k_filter_write<true, true><<<(unsigned) ntiles, FL_THREADS, 0, s>>>((const char*) in->data, in->n, w, P, P16,
				offs, (char*) out, vec);
	else if (vec && w == 16)
		k_filter_write<true, false><<<(unsigned) ntiles, FL_THREADS, 0, s>>>((const char*) in->data, in->n, w, P, P16,
				offs, (char*) out, vec);
	else
		k_filter_write<false, false><<<(unsigned) ntiles, FL_THREADS, 0, s>>>((const char*) in->data, in->n, w, P, P16,
				offs, (char*) out, vec);
	PG_LAUNCHED(ctx);
	uint64_t total = 0;
	PG_CUDA(ctx, cudaMemcpyAsync(&total, offs + ntiles, 8, cudaMemcpyDeviceToHost, s));
	pg_free_async(ctx, s, offs);
	pg_free_async(ctx, s, chars);
	if ((rc = pg_check_status(ctx, s, "pg_filter"))) return rc;
	*n_out = total;
	return PG_OK;
}

struct ProjCols {
	int n;
	uint16_t src[HJ_PROJ_MAX];    // word offset in the input tuple
	uint8_t words[HJ_PROJ_MAX];
	uint32_t ow;                  // output words
};

// Tiles of up to PJ_TILE_WORDS input words (whole tuples): the block loads
// the tile with consecutive threads on consecutive 16-byte vectors (or words
// when the tuple is not a multiple of 16 bytes), then writes the tile's output
// the same way, each output word read from shared memory through the
// output-word -> input-word map.
#define PJ_TILE_WORDS 8192
#define PJ_MAX_WORDS 32
__global__ void __launch_bounds__(256)
k_project(const uint32_t* __restrict__ in, uint64_t n, uint32_t iw, const ProjCols pc,
		uint32_t* __restrict__ out, bool vin, bool vout)
{
	__shared__ uint4 tile4[PJ_TILE_WORDS / 4];
	__shared__ uint16_t map[PJ_MAX_WORDS * 2];
	uint32_t* tile = reinterpret_cast<uint32_t*>(tile4);
	if (threadIdx.x == 0) {
		uint32_t k = 0;
		for (int c = 0; c < pc.n; ++c)
			for (uint32_t q = 0; q < pc.words[c]; ++q) map[k++] = (uint16_t) (pc.src[c] + q);
	}
	__syncthreads();
	const uint32_t ow = pc.ow;
	const uint32_t rpt = PJ_TILE_WORDS / iw;
	const uint64_t ntiles = pg_div_up(n, rpt);
	for (uint64_t tl = blockIdx.x; tl < ntiles; tl += gridDim.x) {
		const uint64_t t0 = tl * rpt;
		const uint32_t rows = (uint32_t) pg_min64(rpt, n - t0);
		const uint32_t iwords = rows * iw, owords = rows * ow;
		const uint32_t* src = in + t0 * iw;
		if (vin) {
			const uint4* s4 = reinterpret_cast<const uint4*>(src);
			for (uint32_t i = threadIdx.x; i < iwords / 4; i += blockDim.x) tile4[i] = __ldcs(s4 + i);
		} else {
			for (uint32_t i = threadIdx.x; i < iwords; i += blockDim.x) tile[i] = __ldcs(src + i);
		}
		__syncthreads();
		uint32_t* dst = out + t0 * ow;
		if (vout) {
			uint4* d4 = reinterpret_cast<uint4*>(dst);
			for (uint32_t i = threadIdx.x; i < owords / 4; i += blockDim.x) {
				const uint32_t t = 4 * i / ow, k = 4 * i - t * ow;
				const uint32_t* r = tile + t * iw;
				__stcs(d4 + i, make_uint4(r[map[k]], r[map[k + 1]], r[map[k + 2]], r[map[k + 3]]));
			}
		} else {
			for (uint32_t i = threadIdx.x; i < owords; i += blockDim.x) {
				const uint32_t t = i / ow, k = i - t * ow;
				__stcs(dst + i, tile[t * iw + map[k]]);
			}
		}
		__syncthreads();
	}
}

// Tuples wider than PJ_MAX_WORDS words: one thread per tuple.
__global__ void k_project_wide(const uint32_t* __restrict__ in, uint64_t n, uint32_t iw, const ProjCols pc,
		uint32_t* __restrict__ out)
{
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
		const uint32_t* t = in + i * iw;
		uint32_t* o = out + i * pc.ow;
		uint32_t k = 0;
		#pragma unroll
		for (int c = 0; c < HJ_PROJ_MAX; ++c) {
			if (c >= pc.n) break;
			for (uint32_t q = 0; q < pc.words[c]; ++q) o[k++] = __ldcs(t + pc.src[c] + q);
		}
	}
}

extern "C" int pg_project(pg_ctx* ctx, pg_stream stream, const pg_rel* in, const pg_col* cols, int ncols, void* out)
{
	if (!ctx || !in) return pg_fail(ctx, PG_ERR_ARG, "pg_project: null argument");
	if (ncols < 1 || ncols > HJ_PROJ_MAX || !cols) return pg_fail(ctx, PG_ERR_ARG, "pg_project: 1..16 columns");
	if (in->width == 0 || (in->width & 3)) return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_project: tuple width must be a multiple of 4");
	if (in->n && (!in->data || !out)) return pg_fail(ctx, PG_ERR_ARG, "pg_project: null data");
	if (in->n && ((reinterpret_cast<uintptr_t>(in->data) | reinterpret_cast<uintptr_t>(out)) & 3))
		return pg_fail(ctx, PG_ERR_ARG, "pg_project: data must be 4-byte aligned");
	ProjCols pc;
	pc.n = ncols; pc.ow = 0;
	for (int c = 0; c < ncols; ++c) {
		if ((cols[c].off & 3) || (cols[c].bytes & 3) || cols[c].bytes == 0 || cols[c].off + cols[c].bytes > in->width)
			return pg_fail(ctx, PG_ERR_ARG, "pg_project: columns must be 4-byte multiples inside the tuple");
		pc.src[c] = (uint16_t) (cols[c].off / 4);
		pc.words[c] = (uint8_t) (cols[c].bytes / 4);
		pc.ow += cols[c].bytes / 4;
	}
	if (in->n == 0) return PG_OK;
	cudaStream_t s = (cudaStream_t) stream;
	const uint32_t iw = in->width / 4;
	if (iw <= PJ_MAX_WORDS && pc.ow <= 2 * PJ_MAX_WORDS) {
		// 32 KB of tile per block: up to 6 blocks per SM. Vectors when the
		// tuples (and so every tile) start on 16-byte boundaries.
		const bool vin = (iw & 3) == 0 && (reinterpret_cast<uintptr_t>(in->data) & 15) == 0;
		const bool vout = (pc.ow & 3) == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0;
		const uint64_t ntiles = pg_div_up(in->n, PJ_TILE_WORDS / iw);
		const int grid = (int) std::min<uint64_t>(ntiles, (uint64_t) ctx->sm_count * 6);
		k_project<<<grid, 256, 0, s>>>((const uint32_t*) in->data, in->n, iw, pc, (uint32_t*) out, vin, vout);
	} else {
		const int grid = (int) std::min<uint64_t>(pg_div_up(in->n, 256), (uint64_t) ctx->sm_count * 16);
		k_project_wide<<<grid, 256, 0, s>>>((const uint32_t*) in->data, in->n, iw, pc, (uint32_t*) out);
	}
	PG_LAUNCHED(ctx);
	return pg_check_status(ctx, s, "pg_project");
}
