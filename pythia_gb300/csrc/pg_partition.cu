// Stable range/radix partitioning on sm_103a.
//
// Replaces PartitionOp's three phases (operators/partition.cpp:166-359):
// histogram (copySourceIntoPageAndPopulateHistogram, :166-200), per-partition
// prefix over workers (:292-307) and the stable scatter (repartition,
// :250-268). The reference's "workers" become CTAs: CTA c owns a contiguous
// chunk of the input, so the output order within a partition is input order,
// exactly what the reference produces when its threads read consecutive
// slices.
//
// Pass 1 (k_part_hist) counts tuples per (bucket, CTA). An exclusive scan over
// the bucket-major counts gives every CTA its first output slot per bucket.
// Pass 2 (k_part_scatter) streams the chunk again in tiles staged in shared
// memory by bulk copies (cp.async.bulk + mbarrier, double-buffered), ranks
// tuples within the tile per bucket (per-warp ballots over the bucket bits +
// per-warp counters, which keeps the order stable), and writes each tile out grouped by bucket so a
// warp's stores go to consecutive addresses of one partition
// (write-combining through shared memory).
#include "pg_internal.cuh"
#include <algorithm>

#define PART_MAX_BUCKETS 4096
#define PART_TILE_BYTES (20 * 1024)     // measured best: 4 CTAs per SM

// Bucket of the key at p: the radix function (parammodulo, the sort's
// digits) inlined when FN says so, else the general bucket function.
#define PART_FN_ANY (-1)
template <int FN>
__device__ __forceinline__ uint32_t part_bucket(const pg_hashfn& f, const char* p, uint32_t kbytes)
{
	if (FN == PG_FN_PARAMMODULO) {
		const int64_t v = pg_load_key(p, kbytes);
		return (uint32_t) (((v - f.min) & f.k) >> f.skipbits);
	}
	if (FN == PG_FN_MIXRADIX) return (uint32_t) (pg_mix64((uint64_t) pg_load_key(p, kbytes)) >> f.skipbits);
	return pg_hash_field(f, p, kbytes);
}

template <int FN>
__global__ void k_part_hist(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t koff,
		uint32_t kbytes, pg_hashfn f, uint32_t tile, uint64_t tiles_per_cta,
		uint64_t* __restrict__ counts, uint32_t G, int* __restrict__ status)
{
	extern __shared__ uint32_t hist[];
	const uint32_t B = f.nbuckets;
	for (uint32_t b = threadIdx.x; b < B; b += blockDim.x) hist[b] = 0;
	__syncthreads();
	uint64_t lo = (uint64_t) blockIdx.x * tiles_per_cta * tile;
	uint64_t hi = std::min<uint64_t>(n, lo + tiles_per_cta * tile);
	bool bad = false;
	for (uint64_t i = lo + threadIdx.x; i < hi; i += blockDim.x) {
		uint32_t b = part_bucket<FN>(f, in + i * W + koff, kbytes);
		if (b < B) atomicAdd(&hist[b], 1u); else bad = true;
	}
	if (bad) pg_set_status(status, PG_ERR_ARG);
	__syncthreads();
	for (uint32_t b = threadIdx.x; b < B; b += blockDim.x)
		counts[(uint64_t) b * G + blockIdx.x] = hist[b];
}

// Copies `bytes` from global to shared with 4-byte words (fallback path for
// tiles a bulk copy cannot take: unaligned base or ragged tail).
__device__ __forceinline__ void part_copy_words(uint32_t* dst, const uint32_t* src, uint32_t words)
{
	for (uint32_t i = threadIdx.x; i < words; i += blockDim.x) dst[i] = src[i];
}

// NBITS > 0: the bucket index has exactly NBITS bits (ranking loop unrolled).
template <int NW, int FN, int NBITS>
__global__ void __launch_bounds__(NW * 32)
k_part_scatter(const char* __restrict__ in, uint64_t n, uint32_t W, uint32_t koff, uint32_t kbytes,
		pg_hashfn f, uint32_t tile, uint64_t tiles_per_cta, const uint64_t* __restrict__ offs,
		uint32_t G, char* __restrict__ out, bool bulk_ok, int* __restrict__ status)
{
	extern __shared__ __align__(128) unsigned char smem[];
	const uint32_t B = f.nbuckets;
	const uint32_t tile_bytes = tile * W;
	unsigned char* buf0 = smem;
	unsigned char* buf1 = smem + tile_bytes;
	uint16_t* cnt = reinterpret_cast<uint16_t*>(smem + 2 * tile_bytes);        // [NW][B]
	uint32_t* tstart = reinterpret_cast<uint32_t*>(cnt + NW * B);               // [B]
	uint32_t* delta = tstart + B;                                                // [B]
	uint32_t* running = delta + B;                                               // [B]
	uint16_t* inv = reinterpret_cast<uint16_t*>(running + B);                   // [tile]
	uint16_t* bkt = inv + tile;                                                  // [tile]
	uint64_t* bar = reinterpret_cast<uint64_t*>(
			(reinterpret_cast<uintptr_t>(bkt + tile) + 15) & ~uintptr_t(15));     // [2]
	__shared__ uint32_t warp_sums[32];
	__shared__ uint32_t carry;

	const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
	const uint32_t nbits = NBITS > 0 ? NBITS : (B > 1 ? 32 - __clz(B - 1) : 0);
	const uint64_t first = (uint64_t) blockIdx.x * tiles_per_cta;
	const uint64_t ntiles_total = pg_div_up(n, tile);
	const uint64_t last = std::min<uint64_t>(ntiles_total, first + tiles_per_cta);
	if (first >= last) return;

	for (uint32_t b = tid; b < B; b += blockDim.x) running[b] = (uint32_t) offs[(uint64_t) b * G + blockIdx.x];
	for (uint32_t i = tid; i < NW * B; i += blockDim.x) cnt[i] = 0;
	if (tid == 0) { pg_mbar_init(&bar[0], 1); pg_mbar_init(&bar[1], 1); pg_fence_mbar_init(); }
	__syncthreads();

	// Issue the load of tile t into buffer (t & 1). Bulk copies only for
	// whole, 16-byte multiple tiles; the rest are copied by the threads.
	auto tile_rows = [&](uint64_t t) -> uint32_t {
		return (uint32_t) std::min<uint64_t>(tile, n - t * tile);
	};
	auto issue = [&](uint64_t t) {
		uint32_t rows = tile_rows(t);
		uint32_t bytes = rows * W;
		unsigned char* dst = (t & 1) ? buf1 : buf0;
		const char* src = in + t * (uint64_t) tile * W;
		if (bulk_ok && (bytes & 15) == 0) {
			if (tid == 0) {
				pg_mbar_expect_tx(&bar[t & 1], bytes);
				pg_bulk_g2s(dst, src, bytes, &bar[t & 1]);
			}
			return true;
		}
		return false;
	};
	uint32_t phase[2] = {0, 0};
	const uint32_t spin = pg_spin_knob(status);
	bool bulk_pending = issue(first);

	for (uint64_t t = first; t < last; ++t) {
		const uint32_t rows = tile_rows(t);
		unsigned char* cur = (t & 1) ? buf1 : buf0;
		if (bulk_pending) {
			if (!pg_mbar_wait_timed(&bar[t & 1], phase[t & 1], spin, status)) return;
			phase[t & 1] ^= 1;
		} else {
			part_copy_words(reinterpret_cast<uint32_t*>(cur),
					reinterpret_cast<const uint32_t*>(in + t * (uint64_t) tile * W), rows * W / 4);
		}
		__syncthreads();
		// Prefetch the next tile into the other buffer while this one is ranked.
		bool next_bulk = false;
		if (t + 1 < last) next_bulk = issue(t + 1);

		// (1) rank within the tile: warp w owns rows [w*sub, (w+1)*sub).
		// Lanes with the same bucket are found with one ballot per bucket
		// bit (the bucket index has nbits bits): cheaper than a match over
		// 32-bit values, with the same peer masks.
		const uint32_t sub = tile / NW;
		uint16_t* mycnt = cnt + warp * B;
		for (uint32_t it = 0; it < sub; it += 32) {
			uint32_t p = warp * sub + it + lane;
			bool valid = p < rows;
			uint32_t b = valid ? part_bucket<FN>(f, reinterpret_cast<const char*>(cur) + (uint64_t) p * W + koff, kbytes) : 0u;
			if (valid && b >= B) { pg_set_status(status, PG_ERR_ARG); b = 0; }
			uint32_t peers = __ballot_sync(0xffffffffu, valid);
			#pragma unroll
			for (uint32_t k = 0; k < (NBITS > 0 ? (uint32_t) NBITS : nbits); ++k) {
				const bool on = (b >> k) & 1u;
				const uint32_t m = __ballot_sync(0xffffffffu, on);
				peers &= on ? m : ~m;
			}
			uint32_t leader = __ffs(peers) - 1;
			uint32_t below = peers & ((1u << lane) - 1);
			uint32_t old = 0;
			if (valid && lane == leader) {
				old = mycnt[b];
				mycnt[b] = (uint16_t) (old + __popc(peers));
			}
			old = __shfl_sync(0xffffffffu, old, leader);
			if (valid) {
				bkt[p] = (uint16_t) b;
				inv[p] = (uint16_t) (old + __popc(below));   // rank within warp sub-tile, for now
			}
			__syncwarp();
		}
		__syncthreads();
		// (2) per bucket: warp prefixes, tile totals, and a scan over buckets
		// for each bucket's first row of the grouped tile.
		if (tid == 0) carry = 0;
		__syncthreads();
		for (uint32_t b0 = 0; b0 < B; b0 += blockDim.x) {
			uint32_t b = b0 + tid;
			uint32_t tot = 0;
			if (b < B) {
				#pragma unroll 4
				for (int w = 0; w < NW; ++w) {
					uint32_t c = cnt[w * B + b];
					cnt[w * B + b] = (uint16_t) tot;
					tot += c;
				}
			}
			// block exclusive scan of tot
			uint32_t x = tot;
			#pragma unroll
			for (int o = 1; o < 32; o <<= 1) {
				uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
				if (lane >= o) x += y;
			}
			if (lane == 31) warp_sums[warp] = x;
			__syncthreads();
			if (warp == 0) {
				uint32_t v = lane < NW ? warp_sums[lane] : 0, vv = v;
				#pragma unroll
				for (int o = 1; o < 32; o <<= 1) {
					uint32_t y = __shfl_up_sync(0xffffffffu, vv, o);
					if (lane >= o) vv += y;
				}
				if (lane < NW) warp_sums[lane] = vv - v;
				if (lane == NW - 1) warp_sums[31] = vv;
			}
			__syncthreads();
			if (b < B) {
				const uint32_t ts = carry + x - tot + warp_sums[warp];
				tstart[b] = ts;
				// Output row of grouped slot s of bucket b: running[b] + (s - ts),
				// kept as one word mod 2^32 (rows stay below 2^32).
				delta[b] = running[b] - ts;
				running[b] += tot;
			}
			__syncthreads();
			if (tid == 0) carry += warp_sums[31];
			__syncthreads();
		}
		// (3) grouped slot of every row, recorded as the permutation
		// slot -> row.
		uint16_t* perm = reinterpret_cast<uint16_t*>(bar + 2);
		for (uint32_t it = 0; it < sub; it += 32) {
			uint32_t p = warp * sub + it + lane;
			if (p < rows) {
				uint32_t b = bkt[p];
				perm[tstart[b] + cnt[warp * B + b] + inv[p]] = (uint16_t) p;
			}
		}
		__syncthreads();
		// (4) write out: slot s of bucket b goes to row delta[b] + s. Threads
		// walk the tile in grouped order so that neighbouring lanes store to
		// neighbouring rows of one partition.
		{
			if (W == 16) {
				for (uint32_t s = tid; s < rows; s += blockDim.x) {
					uint32_t p = perm[s];
					uint32_t b = bkt[p];
					uint64_t dest = (uint32_t) (delta[b] + s);
					uint4 v = reinterpret_cast<const uint4*>(cur)[p];
					pg_st_stream16(out + dest * 16, v);
				}
			} else {
				const uint32_t words = W / 4;
				for (uint32_t e = tid; e < rows * words; e += blockDim.x) {
					uint32_t s = e / words, wd = e - s * words;
					uint32_t p = perm[s];
					uint32_t b = bkt[p];
					uint64_t dest = (uint32_t) (delta[b] + s);
					reinterpret_cast<uint32_t*>(out + dest * W)[wd] =
						reinterpret_cast<const uint32_t*>(cur + (uint64_t) p * W)[wd];
				}
			}
		}
		// (5) reset the counters: step (2) left warp prefixes in every warp's
		// row of each bucket present in the tile. Small tables are cleared
		// whole, large ones only at the buckets this tile used.
		if (NW * B <= 4 * rows) {
			for (uint32_t i = tid; i < NW * B; i += blockDim.x) cnt[i] = 0;
		} else {
			for (uint32_t p = tid; p < rows; p += blockDim.x) {
				uint32_t b = bkt[p];
				#pragma unroll
				for (int w = 0; w < NW; ++w) cnt[w * B + b] = 0;
			}
		}
		__syncthreads();
		bulk_pending = next_bulk;
	}
}

static size_t part_smem_bytes(uint32_t tile, uint32_t W, uint32_t B, int NW)
{
	size_t s = 2 * (size_t) tile * W;          // tile buffers
	s += (size_t) NW * B * 2;                  // per-warp counters
	s += 3 * (size_t) B * 4;                   // tstart, delta, running
	s += 2 * (size_t) tile * 2;                // inv, bkt
	s = (s + 15) & ~size_t(15);
	s += 16;                                   // mbarriers
	s += (size_t) tile * 2;                    // grouped-slot -> row permutation
	return s;
}

extern "C" int pg_partition(pg_ctx* ctx, pg_stream stream, const pg_rel* in,
		const pg_hashcfg* cfg, void* out, uint64_t* offsets)
{
	if (!ctx || !in || !cfg || !offsets) return pg_fail(ctx, PG_ERR_ARG, "pg_partition: null argument");
	pg_hashfn f;
	if (pg_hashfn_derive(cfg, &f)) return pg_fail(ctx, PG_ERR_ARG, "pg_partition: invalid hash configuration");
	int rc = pg_partition_fn(ctx, (cudaStream_t) stream, in, f, out, offsets);
	if (rc) return rc;
	return pg_check_status(ctx, (cudaStream_t) stream, "pg_partition");
}

// Partition by an already derived bucket function; offsets may be null. Does
// not synchronise (the radix sort chains passes on the stream).
int pg_partition_fn(pg_ctx* ctx, cudaStream_t s, const pg_rel* in, const pg_hashfn& f,
		void* out, uint64_t* offsets)
{
	const uint32_t B = f.nbuckets, W = in->width;
	if (B == 0 || B > PART_MAX_BUCKETS)
		return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_partition: at most 4096 buckets in one pass");
	if (W == 0 || (W & 3) || W > 1024)
		return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_partition: tuple width must be a multiple of 4 bytes, at most 1024");
	if (in->key_off + in->key_bytes > W || (in->key_bytes != 4 && in->key_bytes != 8))
		return pg_fail(ctx, PG_ERR_ARG, "pg_partition: key must be a 4- or 8-byte column inside the tuple");
	if (in->n >= (1ull << 32)) return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_partition: at most 2^32-1 tuples");
	const uint64_t n = in->n;
	if (n == 0) {
		if (offsets) PG_CUDA(ctx, cudaMemsetAsync(offsets, 0, (B + 1) * sizeof(uint64_t), s));
		return PG_OK;
	}
	const int NW = B <= 1024 ? 8 : 4;
	const int64_t tb = ctx->tune[PG_TUNE_PARTITION_TILE];
	uint32_t tile = (uint32_t) (tb > 0 ? std::min<int64_t>(65536, std::max<int64_t>(8192, tb)) : PART_TILE_BYTES) / W;
	tile = std::max<uint32_t>(NW * 32, tile / (NW * 32) * (NW * 32));
	const uint64_t ntiles = pg_div_up(n, tile);
	const size_t smem = part_smem_bytes(tile, W, B, NW);
	if (smem > 220 * 1024) return pg_fail(ctx, PG_ERR_UNSUPPORTED, "pg_partition: tile does not fit shared memory");
	int per_sm = (int) std::max<size_t>(1, std::min<size_t>(8, (228 * 1024) / (smem + 1024)));
	uint64_t G = std::min<uint64_t>(ntiles, (uint64_t) ctx->sm_count * per_sm);
	uint64_t tpc = pg_div_up(ntiles, G);
	G = pg_div_up(ntiles, tpc);

	int rc;
	uint64_t* counts = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &counts, (size_t) B * G * 8 + 8))) return rc;
	const bool radix = f.fn == PG_FN_PARAMMODULO, mix = f.fn == PG_FN_MIXRADIX;
	if (radix)
		k_part_hist<PG_FN_PARAMMODULO><<<(unsigned) G, 512, B * sizeof(uint32_t), s>>>((const char*) in->data, n, W,
				in->key_off, in->key_bytes, f, tile, tpc, counts, (uint32_t) G, ctx->d_status);
	else if (mix)
		k_part_hist<PG_FN_MIXRADIX><<<(unsigned) G, 512, B * sizeof(uint32_t), s>>>((const char*) in->data, n, W,
				in->key_off, in->key_bytes, f, tile, tpc, counts, (uint32_t) G, ctx->d_status);
	else
		k_part_hist<PART_FN_ANY><<<(unsigned) G, 512, B * sizeof(uint32_t), s>>>((const char*) in->data, n, W,
				in->key_off, in->key_bytes, f, tile, tpc, counts, (uint32_t) G, ctx->d_status);
	PG_LAUNCHED(ctx);
	if ((rc = pg_scan_u64(ctx, s, counts, (uint64_t) B * G, nullptr))) return rc;
	bool bulk_ok = ((reinterpret_cast<uintptr_t>(in->data) & 15) == 0) && (((uint64_t) tile * W) % 16 == 0);
#define PS_LAUNCH(NWv, FNv, NB) do { \
		PG_CUDA(ctx, cudaFuncSetAttribute(k_part_scatter<NWv, FNv, NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem)); \
		k_part_scatter<NWv, FNv, NB><<<(unsigned) G, NWv * 32, smem, s>>>((const char*) in->data, n, W, in->key_off, \
				in->key_bytes, f, tile, tpc, counts, (uint32_t) G, (char*) out, bulk_ok, ctx->d_status); } while (0)
	// Radix passes (parammodulo) of 256 or 64 buckets and partitions on the
	// top bits of the key hash (mixradix, 32 to 256 buckets) take specialised
	// kernels; everything else the general one.
	if (NW == 8 && radix && B == 256) PS_LAUNCH(8, PG_FN_PARAMMODULO, 8);
	else if (NW == 8 && radix && B == 64) PS_LAUNCH(8, PG_FN_PARAMMODULO, 6);
	else if (NW == 8 && mix && B == 256) PS_LAUNCH(8, PG_FN_MIXRADIX, 8);
	else if (NW == 8 && mix && B == 128) PS_LAUNCH(8, PG_FN_MIXRADIX, 7);
	else if (NW == 8 && mix && B == 64) PS_LAUNCH(8, PG_FN_MIXRADIX, 6);
	else if (NW == 8 && mix && B == 32) PS_LAUNCH(8, PG_FN_MIXRADIX, 5);
	else if (NW == 8) PS_LAUNCH(8, PART_FN_ANY, 0);
	else PS_LAUNCH(4, PART_FN_ANY, 0);
#undef PS_LAUNCH
	PG_LAUNCHED(ctx);
	// offsets[b] = first slot of bucket b = scanned count of (b, CTA 0).
	// Strided copy: counts[b*G] for b < B, then n.
	if (offsets) {
		PG_CUDA(ctx, cudaMemcpy2DAsync(offsets, sizeof(uint64_t), counts, G * sizeof(uint64_t),
				sizeof(uint64_t), B, cudaMemcpyDeviceToDevice, s));
		PG_CUDA(ctx, cudaMemcpyAsync(offsets + B, &in->n, sizeof(uint64_t), cudaMemcpyHostToDevice, s));
	}
	pg_free_async(ctx, s, counts);
	return PG_OK;
}
