// Batched uneven joins on sm_103a.
//
// Many independent join + aggregate_count instances (the reference would run
// one HashJoinOp plan per instance under a MergeOp, operators/join.cpp:
// 273-675 with aggregatecount.cpp:37-52 above it) are executed by one build
// launch and one probe launch per size class instead of two launches, a host
// synchronisation and scratch allocations per instance. Work is cut into
// tiles that never straddle instances; each persistent CTA walks the tile
// list, so a 1K-tuple instance and a 32M-tuple instance share the machine
// without per-instance launch overhead. The sequence (table clear, build,
// probe, count copy-out) can be captured once as a CUDA graph and replayed.
//
// An instance whose build keys are unique and whose key range needs no more
// bytes as a bitmap than its hash table would (range / 8 <= 16 * slots) gets a
// presence bitmap: the probe of a count-only PK-FK join then reads one bit
// per probe tuple, and the bitmaps of a wave stay in L2. Other instances get
// their own open-addressing table region (16-byte slots, linear probing from
// an even slot, 32-byte bucket loads on probe) sized by the class's load
// factor. Launch shape (threads per CTA, tile size, CTAs per SM) and load
// factor come from pg_batch_shape, which the autotuner chooses per size
// class.
#include "pg_internal.cuh"
#include <algorithm>
#include <vector>

struct BatchInst {
	const char* R; const char* S;
	uint64_t nR, nS;
	uint64_t table_off;     // hashed: first slot of the instance's table; bitmap: first word
	uint32_t log2cap;
	uint32_t mode;          // 0 hashed table, 1 presence bitmap over keys [kmin, kmin + range)
	long long kmin;
	uint64_t range;
};

struct BatchTile {           // [begin, end) of one side of instance `inst`
	uint32_t inst;
	uint32_t pad;
	uint64_t begin, end;
};

__device__ __forceinline__ uint64_t bt_slot0(int64_t k, uint32_t log2cap)
{
	return (pg_mix64((uint64_t) k) >> (65 - log2cap)) << 1;
}

// Build. Bitmap instances set their keys' bits; a bit found set already (a
// repeated key) or a key outside the range marks the instance in `dup` (the
// prepare-time trial) or fails the batch (a replay whose build side changed
// since prepare: PG_ERR_ARG).
__global__ void k_batch_build(const BatchInst* __restrict__ inst, const BatchTile* __restrict__ tiles,
		uint64_t ntiles, unsigned long long* __restrict__ slots, uint32_t* __restrict__ bits,
		int* __restrict__ dup, bool trial, int* __restrict__ status)
{
	for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
		const BatchTile tl = tiles[t];
		const BatchInst in = inst[tl.inst];
		if (in.mode == 1) {
			bool bad = false;
			for (uint64_t i = tl.begin + threadIdx.x; i < tl.end; i += blockDim.x) {
				const long long k = reinterpret_cast<const long long*>(in.R)[2 * i];
				const unsigned long long d = (unsigned long long) k - (unsigned long long) in.kmin;
				if (d >= in.range) { bad = true; continue; }
				const uint32_t bit = 1u << (d & 31);
				if (atomicOr(&bits[in.table_off + (d >> 5)], bit) & bit) bad = true;
			}
			if (bad) {
				if (trial) dup[tl.inst] = 1;
				else pg_set_status(status, PG_ERR_ARG);
			}
			continue;
		}
		if (trial) continue;        // the trial builds bitmaps only (no slots exist yet)
		unsigned long long* tab = slots + 2 * in.table_off;
		const uint64_t mask = (1ull << in.log2cap) - 1;
		for (uint64_t i = tl.begin + threadIdx.x; i < tl.end; i += blockDim.x) {
			const uint4 tup = reinterpret_cast<const uint4*>(in.R)[i];
			const long long k = (long long) (((uint64_t) tup.y << 32) | tup.x);
			const unsigned long long v = ((unsigned long long) tup.w << 32) | tup.z;
			uint64_t s = bt_slot0(k, in.log2cap), probe = 0;
			for (; probe <= mask; ++probe) {
				const unsigned long long old = atomicCAS(&tab[2 * s], (unsigned long long) PG_EMPTY_KEY,
						(unsigned long long) k);
				if (old == (unsigned long long) PG_EMPTY_KEY) { tab[2 * s + 1] = v; break; }
				s = (s + 1) & mask;
			}
			if (probe > mask) pg_set_status(status, PG_ERR_TABLE_FULL);
		}
	}
}

// Counts, per instance, the probe tuples' matches (duplicates included: the
// probe walks its whole sequence). One atomicAdd per tile and CTA.
template <int ITEMS>
__global__ void k_batch_probe_count(const BatchInst* __restrict__ inst, const BatchTile* __restrict__ tiles,
		uint64_t ntiles, const unsigned long long* __restrict__ slots, const uint32_t* __restrict__ bits,
		unsigned long long* __restrict__ counts)
{
	__shared__ unsigned long long wsum[32];
	const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
	const uint64_t keep = pg_policy_evict_last();
	for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
		const BatchTile tl = tiles[t];
		const BatchInst in = inst[tl.inst];
		const unsigned long long* tab = slots + 2 * in.table_off;
		const uint64_t mask = (1ull << in.log2cap) - 1;
		unsigned long long c = 0;
		if (in.mode == 1) {
			// Presence bitmap: one bit per probe tuple.
			for (uint64_t base = tl.begin; base < tl.end; base += (uint64_t) blockDim.x * ITEMS) {
				uint32_t w[ITEMS];
				uint64_t d[ITEMS];
				#pragma unroll
				for (int j = 0; j < ITEMS; ++j) {
					const uint64_t i = base + (uint64_t) j * blockDim.x + threadIdx.x;
					d[j] = ~0ull; w[j] = 0;
					if (i < tl.end)
						d[j] = (unsigned long long) reinterpret_cast<const long long*>(in.S)[2 * i] - (unsigned long long) in.kmin;
					if (d[j] < in.range) w[j] = __ldg(bits + in.table_off + (d[j] >> 5));
				}
				#pragma unroll
				for (int j = 0; j < ITEMS; ++j) c += d[j] < in.range ? (w[j] >> (d[j] & 31)) & 1 : 0;
			}
		} else
		for (uint64_t base = tl.begin; base < tl.end; base += (uint64_t) blockDim.x * ITEMS) {
			long long key[ITEMS];
			uint64_t slot[ITEMS];
			bool open[ITEMS];
			#pragma unroll
			for (int j = 0; j < ITEMS; ++j) {
				const uint64_t i = base + (uint64_t) j * blockDim.x + threadIdx.x;
				open[j] = i < tl.end;
				key[j] = open[j] ? reinterpret_cast<const long long*>(in.S)[2 * i] : 0;
				slot[j] = bt_slot0(key[j], in.log2cap);
			}
			for (uint64_t round = 0; round <= (mask >> 1); ++round) {
				pg_u64x4 bk[ITEMS];
				bool any = false;
				#pragma unroll
				for (int j = 0; j < ITEMS; ++j)
					if (open[j]) { bk[j] = pg_ld_bucket32(tab + 2 * slot[j], keep); any = true; }
				if (!any) break;
				#pragma unroll
				for (int j = 0; j < ITEMS; ++j) {
					if (!open[j]) continue;
					if ((long long) bk[j].a == key[j]) ++c;
					if (bk[j].a == (unsigned long long) PG_EMPTY_KEY) { open[j] = false; continue; }
					if ((long long) bk[j].c == key[j]) ++c;
					if (bk[j].c == (unsigned long long) PG_EMPTY_KEY) { open[j] = false; continue; }
					slot[j] = (slot[j] + 2) & mask;
				}
			}
		}
		#pragma unroll
		for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
		if (lane == 0) wsum[warp] = c;
		__syncthreads();
		if (threadIdx.x == 0) {
			unsigned long long tot = 0;
			for (int w = 0; w < nwarps; ++w) tot += wsum[w];
			if (tot) atomicAdd(&counts[tl.inst], tot);
		}
		__syncthreads();
	}
}

// Per-instance key minimum and maximum (sign-flipped for unsigned atomics).
// Keys equal to the empty marker never occur in the batch workloads' build
// sides; a key equal to it fails the batch (PG_ERR_UNSUPPORTED) instead of a
// side list per instance.
__global__ void k_batch_minmax(const BatchInst* __restrict__ inst, const BatchTile* __restrict__ tiles,
		uint64_t ntiles, unsigned long long* __restrict__ mm, int* __restrict__ status)
{
	for (uint64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
		const BatchTile tl = tiles[t];
		const BatchInst in = inst[tl.inst];
		unsigned long long lo = ~0ull, hi = 0;
		bool marker = false;
		for (uint64_t i = tl.begin + threadIdx.x; i < tl.end; i += blockDim.x) {
			const long long k = reinterpret_cast<const long long*>(in.R)[2 * i];
			marker |= k == PG_EMPTY_KEY;
			const unsigned long long u = (unsigned long long) k ^ (1ull << 63);
			lo = u < lo ? u : lo;
			hi = u > hi ? u : hi;
		}
		if (marker) pg_set_status(status, PG_ERR_UNSUPPORTED);
		#pragma unroll
		for (int o = 16; o > 0; o >>= 1) {
			const unsigned long long a = __shfl_down_sync(0xffffffffu, lo, o), b = __shfl_down_sync(0xffffffffu, hi, o);
			lo = a < lo ? a : lo;
			hi = b > hi ? b : hi;
		}
		if ((threadIdx.x & 31) == 0) { atomicMin(&mm[2 * tl.inst], lo); atomicMax(&mm[2 * tl.inst + 1], hi); }
	}
}


// Synthetic foreign keys: S[j].key = R[h(seed, j) mod nR].key, payload from
// the same counter hash (SplitMix64 finaliser; multiply-high reduction).
__global__ void k_generate_fk(const char* __restrict__ R, uint64_t nR, uint64_t seed, char* __restrict__ S, uint64_t nS)
{
	for (uint64_t j = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; j < nS;
			j += (uint64_t) gridDim.x * blockDim.x) {
		uint64_t z = seed + (j + 1) * 0x9E3779B97F4A7C15ull;
		z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
		z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
		z ^= z >> 31;
		const uint64_t idx = __umul64hi(z, nR);
		const long long key = reinterpret_cast<const long long*>(R)[2 * idx];
		reinterpret_cast<long long*>(S)[2 * j] = key;
		reinterpret_cast<long long*>(S)[2 * j + 1] = (long long) ((z * 0xD1B54A32D192ED03ull) >> 33);
	}
}

extern "C" int pg_generate_fk(pg_ctx* ctx, pg_stream stream, const void* R, uint64_t nR, uint64_t seed,
		void* S, uint64_t nS)
{
	if (!ctx || (nS && (!R || !S || nR == 0))) return pg_fail(ctx, PG_ERR_ARG, "pg_generate_fk: bad argument");
	if (nS == 0) return PG_OK;
	const int blocks = (int) std::min<uint64_t>(pg_div_up(nS, 256), (uint64_t) ctx->sm_count * 16);
	k_generate_fk<<<blocks, 256, 0, (cudaStream_t) stream>>>((const char*) R, nR, seed, (char*) S, nS);
	PG_LAUNCHED(ctx);
	return PG_OK;
}

// Prepared batch: device descriptors, tile lists and tables; replayable.
struct pg_batch {
	pg_ctx* ctx;
	cudaStream_t stream;
	uint32_t ninst;
	BatchInst* d_inst;
	BatchTile* d_btiles;
	BatchTile* d_ptiles;
	uint64_t nbtiles, nptiles;
	unsigned long long* d_slots;
	uint64_t nslots;
	uint32_t* d_bits;           // presence bitmaps of bitmap instances
	uint64_t nbits_words;
	int* d_dup;                 // per instance: repeated key seen in the prepare trial
	unsigned long long* d_counts;
	pg_batch_shape shape;
	cudaGraphExec_t graph;
	bool has_graph;
};

static int batch_launch(pg_batch* b, cudaStream_t s)
{
	pg_ctx* ctx = b->ctx;
	PG_CUDA(ctx, cudaMemsetAsync(b->d_slots, 0xFF, b->nslots * 16, s));
	PG_CUDA(ctx, cudaMemsetAsync(b->d_bits, 0, b->nbits_words * 4, s));
	PG_CUDA(ctx, cudaMemsetAsync(b->d_counts, 0, b->ninst * 8, s));
	const int per_sm = b->shape.ctas_per_sm > 0 ? b->shape.ctas_per_sm : 4;
	const int threads = b->shape.threads > 0 ? b->shape.threads : 256;
	if (b->nbtiles) {
		const int grid = (int) std::min<uint64_t>(b->nbtiles, (uint64_t) ctx->sm_count * per_sm);
		k_batch_build<<<grid, threads, 0, s>>>(b->d_inst, b->d_btiles, b->nbtiles, b->d_slots, b->d_bits, b->d_dup,
				false, ctx->d_status);
		PG_LAUNCHED(ctx);
	}
	if (b->nptiles) {
		const int grid = (int) std::min<uint64_t>(b->nptiles, (uint64_t) ctx->sm_count * per_sm);
		switch (b->shape.items) {
		case 1: k_batch_probe_count<1><<<grid, threads, 0, s>>>(b->d_inst, b->d_ptiles, b->nptiles, b->d_slots, b->d_bits, b->d_counts); break;
		case 2: k_batch_probe_count<2><<<grid, threads, 0, s>>>(b->d_inst, b->d_ptiles, b->nptiles, b->d_slots, b->d_bits, b->d_counts); break;
		case 8: k_batch_probe_count<8><<<grid, threads, 0, s>>>(b->d_inst, b->d_ptiles, b->nptiles, b->d_slots, b->d_bits, b->d_counts); break;
		default: k_batch_probe_count<4><<<grid, threads, 0, s>>>(b->d_inst, b->d_ptiles, b->nptiles, b->d_slots, b->d_bits, b->d_counts); break;
		}
		PG_LAUNCHED(ctx);
	}
	return PG_OK;
}

extern "C" int pg_batch_prepare(pg_ctx* ctx, pg_stream stream, const pg_batch_item* items, uint32_t n,
		const pg_batch_shape* shape, pg_batch** out)
{
	if (!ctx || !out || (n && !items)) return pg_fail(ctx, PG_ERR_ARG, "pg_batch_prepare: null argument");
	pg_batch_shape sh = {256, 4, 4096, 4, 2, 0};
	if (shape) sh = *shape;
	if (sh.threads != 128 && sh.threads != 256 && sh.threads != 512) sh.threads = 256;
	if (sh.items != 1 && sh.items != 2 && sh.items != 4 && sh.items != 8) sh.items = 4;
	if (sh.tile < 256) sh.tile = 4096;
	if (sh.load_inverse < 2) sh.load_inverse = 2;
	cudaStream_t s = (cudaStream_t) stream;
	std::vector<BatchInst> inst(n);
	std::vector<BatchTile> bt, pt;
	uint64_t slots = 0;
	for (uint32_t i = 0; i < n; ++i) {
		const pg_batch_item& it = items[i];
		if ((it.nR && !it.R) || (it.nS && !it.S))
			return pg_fail(ctx, PG_ERR_ARG, "pg_batch_prepare: null relation");
		if (((reinterpret_cast<uintptr_t>(it.R) | reinterpret_cast<uintptr_t>(it.S)) & 15))
			return pg_fail(ctx, PG_ERR_ARG, "pg_batch_prepare: relations must be 16-byte aligned");
		uint32_t lg = 6;
		while ((1ull << lg) < (uint64_t) sh.load_inverse * it.nR) ++lg;
		inst[i] = BatchInst{(const char*) it.R, (const char*) it.S, it.nR, it.nS, slots, lg, 0, 0, 0};
		slots += 1ull << lg;
		for (uint64_t b = 0; b < it.nR; b += sh.tile) bt.push_back(BatchTile{i, 0, b, std::min<uint64_t>(it.nR, b + sh.tile)});
		for (uint64_t b = 0; b < it.nS; b += sh.tile) pt.push_back(BatchTile{i, 0, b, std::min<uint64_t>(it.nS, b + sh.tile)});
	}
	pg_batch* bb = new pg_batch();
	bb->ctx = ctx; bb->stream = s; bb->ninst = n; bb->shape = sh;
	bb->nbtiles = bt.size(); bb->nptiles = pt.size(); bb->nslots = std::max<uint64_t>(slots, 1);
	bb->has_graph = false;
	bb->nbits_words = 1;
	int rc = PG_OK;
	cudaError_t e;
	if ((e = cudaMalloc(&bb->d_inst, std::max<size_t>(1, n) * sizeof(BatchInst))) ||
			(e = cudaMalloc(&bb->d_btiles, std::max<size_t>(1, bt.size()) * sizeof(BatchTile))) ||
			(e = cudaMalloc(&bb->d_ptiles, std::max<size_t>(1, pt.size()) * sizeof(BatchTile))) ||
			(e = cudaMalloc(&bb->d_counts, std::max<size_t>(1, n) * 8)) ||
			(e = cudaMalloc(&bb->d_dup, std::max<size_t>(1, n) * sizeof(int)))) {
		rc = pg_cuda_fail(ctx, e, "pg_batch_prepare: cudaMalloc");
		pg_batch_free(ctx, bb);
		return rc;
	}
	// Layout choice: per-instance key ranges (one pass over the build sides);
	// instances whose bitmap is no larger than their hash table try the
	// bitmap, and a trial build drops those with repeated keys back to the
	// hash table.
	if (n && !bt.empty()) {
		unsigned long long* mm = nullptr;
		if ((e = cudaMalloc(&mm, 16 * (size_t) n))) { pg_batch_free(ctx, bb); return pg_cuda_fail(ctx, e, "pg_batch_prepare: cudaMalloc"); }
		std::vector<unsigned long long> init(2 * (size_t) n);
		for (uint32_t i = 0; i < n; ++i) { init[2 * i] = ~0ull; init[2 * i + 1] = 0; }
		PG_CUDA(ctx, cudaMemcpyAsync(mm, init.data(), 16 * (size_t) n, cudaMemcpyHostToDevice, s));
		PG_CUDA(ctx, cudaMemcpyAsync(bb->d_inst, inst.data(), n * sizeof(BatchInst), cudaMemcpyHostToDevice, s));
		PG_CUDA(ctx, cudaMemcpyAsync(bb->d_btiles, bt.data(), bt.size() * sizeof(BatchTile), cudaMemcpyHostToDevice, s));
		k_batch_minmax<<<(int) std::min<uint64_t>(bt.size(), (uint64_t) ctx->sm_count * 8), 256, 0, s>>>(
				bb->d_inst, bb->d_btiles, bt.size(), mm, ctx->d_status);
		PG_LAUNCHED(ctx);
		PG_CUDA(ctx, cudaMemcpyAsync(init.data(), mm, 16 * (size_t) n, cudaMemcpyDeviceToHost, s));
		PG_CUDA(ctx, cudaStreamSynchronize(s));
		cudaFree(mm);
		uint64_t words = 0;
		for (uint32_t i = 0; i < n; ++i) {
			if (inst[i].nR == 0) continue;
			const long long kmin = (long long) (init[2 * i] ^ (1ull << 63));
			const long long kmax = (long long) (init[2 * i + 1] ^ (1ull << 63));
			const uint64_t range = (uint64_t) kmax - (uint64_t) kmin + 1;
			if (range == 0 || range > (1ull << 32) || range / 8 > (1ull << inst[i].log2cap) * 16) continue;
			inst[i].mode = 1; inst[i].kmin = kmin; inst[i].range = range; inst[i].table_off = words;
			words += pg_div_up(range, 32);
		}
		bb->nbits_words = std::max<uint64_t>(words, 1);
		if ((e = cudaMalloc(&bb->d_bits, bb->nbits_words * 4))) { pg_batch_free(ctx, bb); return pg_cuda_fail(ctx, e, "pg_batch_prepare: cudaMalloc"); }
		if (words) {
			PG_CUDA(ctx, cudaMemcpyAsync(bb->d_inst, inst.data(), n * sizeof(BatchInst), cudaMemcpyHostToDevice, s));
			PG_CUDA(ctx, cudaMemsetAsync(bb->d_bits, 0, bb->nbits_words * 4, s));
			PG_CUDA(ctx, cudaMemsetAsync(bb->d_dup, 0, n * sizeof(int), s));
			k_batch_build<<<(int) std::min<uint64_t>(bt.size(), (uint64_t) ctx->sm_count * 8), 256, 0, s>>>(
					bb->d_inst, bb->d_btiles, bt.size(), nullptr, bb->d_bits, bb->d_dup, true, ctx->d_status);
			PG_LAUNCHED(ctx);
			std::vector<int> dup(n);
			PG_CUDA(ctx, cudaMemcpyAsync(dup.data(), bb->d_dup, n * sizeof(int), cudaMemcpyDeviceToHost, s));
			PG_CUDA(ctx, cudaStreamSynchronize(s));
			for (uint32_t i = 0; i < n; ++i)
				if (dup[i] && inst[i].mode == 1) { inst[i].mode = 0; inst[i].kmin = 0; inst[i].range = 0; }
		}
	} else if ((e = cudaMalloc(&bb->d_bits, 4))) {
		pg_batch_free(ctx, bb); return pg_cuda_fail(ctx, e, "pg_batch_prepare: cudaMalloc");
	}
	// Hash-table slots for the instances left on the hashed layout.
	slots = 0;
	for (uint32_t i = 0; i < n; ++i) {
		if (inst[i].mode == 1) continue;
		inst[i].table_off = slots;
		slots += 1ull << inst[i].log2cap;
	}
	bb->nslots = std::max<uint64_t>(slots, 1);
	if ((e = cudaMalloc(&bb->d_slots, bb->nslots * 16))) {
		rc = pg_cuda_fail(ctx, e, "pg_batch_prepare: cudaMalloc");
		pg_batch_free(ctx, bb);
		return rc;
	}
	if (n) PG_CUDA(ctx, cudaMemcpyAsync(bb->d_inst, inst.data(), n * sizeof(BatchInst), cudaMemcpyHostToDevice, s));
	if (!bt.empty()) PG_CUDA(ctx, cudaMemcpyAsync(bb->d_btiles, bt.data(), bt.size() * sizeof(BatchTile), cudaMemcpyHostToDevice, s));
	if (!pt.empty()) PG_CUDA(ctx, cudaMemcpyAsync(bb->d_ptiles, pt.data(), pt.size() * sizeof(BatchTile), cudaMemcpyHostToDevice, s));
	if ((rc = pg_check_status(ctx, s, "pg_batch_prepare"))) {
		pg_batch_free(ctx, bb);
		return pg_fail(ctx, rc, "pg_batch_prepare: a build key equals -1 (not supported in batches)");
	}
	if (sh.use_graph) {
		// Capture clear + build + probe once; pg_batch_run replays it.
		cudaGraph_t g;
		if ((e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal))) { pg_batch_free(ctx, bb); return pg_cuda_fail(ctx, e, "cudaStreamBeginCapture"); }
		rc = batch_launch(bb, s);
		e = cudaStreamEndCapture(s, &g);
		if (rc || e) { pg_batch_free(ctx, bb); return rc ? rc : pg_cuda_fail(ctx, e, "cudaStreamEndCapture"); }
		e = cudaGraphInstantiate(&bb->graph, g, 0);
		cudaGraphDestroy(g);
		if (e) { pg_batch_free(ctx, bb); return pg_cuda_fail(ctx, e, "cudaGraphInstantiate"); }
		bb->has_graph = true;
	}
	*out = bb;
	return PG_OK;
}

extern "C" int pg_batch_run(pg_ctx* ctx, pg_batch* b, uint64_t* counts_host)
{
	if (!ctx || !b) return pg_fail(ctx, PG_ERR_ARG, "pg_batch_run: null argument");
	int rc;
	if (b->has_graph) {
		PG_CUDA(ctx, cudaGraphLaunch(b->graph, b->stream));
		g_kernel_launches.fetch_add((b->nbtiles ? 1 : 0) + (b->nptiles ? 1 : 0));
	} else if ((rc = batch_launch(b, b->stream))) return rc;
	if (counts_host && b->ninst)
		PG_CUDA(ctx, cudaMemcpyAsync(counts_host, b->d_counts, b->ninst * 8, cudaMemcpyDeviceToHost, b->stream));
	return pg_check_status(ctx, b->stream, "pg_batch_run");
}

extern "C" int pg_batch_free(pg_ctx* ctx, pg_batch* b)
{
	if (!b) return PG_OK;
	cudaStreamSynchronize(b->stream);
	if (b->has_graph) cudaGraphExecDestroy(b->graph);
	cudaFree(b->d_inst); cudaFree(b->d_btiles); cudaFree(b->d_ptiles);
	cudaFree(b->d_slots); cudaFree(b->d_counts); cudaFree(b->d_bits); cudaFree(b->d_dup);
	delete b;
	(void) ctx;
	return PG_OK;
}

// ---------------------------------------------------------------------------
// Launch-shape autotuner: every candidate shape is prepared on the caller's
// instances, replayed once to warm up, then timed `repeats` times with CUDA
// events on the batch's stream; the fastest shape wins. Shapes change speed,
// never counts, so the sweep needs no checking beyond the status word.
// ---------------------------------------------------------------------------
extern "C" int pg_autotune_batch(pg_ctx* ctx, pg_stream stream, const pg_batch_item* items, uint32_t n,
		const pg_batch_shape* shapes, uint32_t n_shapes, int repeats, uint32_t* best, double* ms_out)
{
	if (!ctx || !shapes || !n_shapes || !best || (n && !items) || repeats < 1)
		return pg_fail(ctx, PG_ERR_ARG, "pg_autotune_batch: bad argument");
	cudaEvent_t e0, e1;
	PG_CUDA(ctx, cudaEventCreate(&e0));
	PG_CUDA(ctx, cudaEventCreate(&e1));
	double best_ms = 1e300;
	*best = 0;
	int rc = PG_OK;
	for (uint32_t k = 0; k < n_shapes && rc == PG_OK; ++k) {
		pg_batch* b = nullptr;
		if ((rc = pg_batch_prepare(ctx, stream, items, n, &shapes[k], &b))) break;
		double mine = 1e300;
		rc = pg_batch_run(ctx, b, nullptr);
		for (int r = 0; r < repeats && rc == PG_OK; ++r) {
			cudaEventRecord(e0, b->stream);
			if ((rc = pg_batch_run(ctx, b, nullptr))) break;
			cudaEventRecord(e1, b->stream);
			if (cudaEventSynchronize(e1) != cudaSuccess) { rc = pg_cuda_fail(ctx, cudaGetLastError(), "pg_autotune_batch"); break; }
			float ms = 0.f;
			cudaEventElapsedTime(&ms, e0, e1);
			mine = std::min(mine, (double) ms);
		}
		pg_batch_free(ctx, b);
		if (ms_out) ms_out[k] = mine;
		if (rc == PG_OK && mine < best_ms) { best_ms = mine; *best = k; }
	}
	cudaEventDestroy(e0);
	cudaEventDestroy(e1);
	return rc;
}

// ---------------------------------------------------------------------------
// Zipf foreign keys on the device (rejection-inversion, Hormann & Derflinger
// 1996): rank k in [1, n] with P(k) ~ k^-s, drawn from a counter hash of
// (seed, j, attempt); s = 0 draws ranks uniformly. Dec payload uniform in
// [0, vmax).
// ---------------------------------------------------------------------------
struct ZipfParams { double s, hx1, hn, sx; uint64_t n; };

__host__ __device__ static inline double zf_h2(double t) { return fabs(t) > 1e-8 ? expm1(t) / t : 1.0 + t * 0.5 * (1.0 + t / 3.0); }
__host__ __device__ static inline double zf_h1(double t) { return fabs(t) > 1e-8 ? log1p(t) / t : 1.0 - t * (0.5 - t / 3.0); }
__host__ __device__ static inline double zf_H(double s, double x) { const double lx = log(x); return zf_h2((1.0 - s) * lx) * lx; }
__host__ __device__ static inline double zf_Hinv(double s, double u) { return exp(zf_h1((1.0 - s) * u) * u); }
__host__ __device__ static inline double zf_h(double s, double x) { return exp(-s * log(x)); }

__device__ __forceinline__ uint64_t zf_hash(uint64_t seed, uint64_t j, uint64_t a)
{
	uint64_t z = seed + (j + 1) * 0x9E3779B97F4A7C15ull + a * 0xD1B54A32D192ED03ull;
	z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
	z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
	return z ^ (z >> 31);
}

__global__ void k_generate_zipf_fk(const char* __restrict__ R, ZipfParams zp, uint64_t seed,
		char* __restrict__ S, uint64_t nS, double vmax)
{
	for (uint64_t j = blockIdx.x * (uint64_t) blockDim.x + threadIdx.x; j < nS;
			j += (uint64_t) gridDim.x * blockDim.x) {
		uint64_t k = 1;
		if (zp.s == 0.0) {
			k = __umul64hi(zf_hash(seed, j, 0), zp.n) + 1;
		} else {
			for (uint64_t a = 0; a < 64; ++a) {
				const double u01 = (double) (zf_hash(seed, j, a) >> 11) * 0x1.0p-53;
				const double u = zp.hn + u01 * (zp.hx1 - zp.hn);
				const double x = zf_Hinv(zp.s, u);
				double kd = floor(x + 0.5);
				kd = kd < 1.0 ? 1.0 : (kd > (double) zp.n ? (double) zp.n : kd);
				k = (uint64_t) kd;
				if (kd - x <= zp.sx || u >= zf_H(zp.s, kd + 0.5) - zf_h(zp.s, kd)) break;
			}
		}
		const long long key = reinterpret_cast<const long long*>(R)[2 * (k - 1)];
		const double v = (double) (zf_hash(seed ^ 0x5A5A5A5Aull, j, 99) >> 11) * 0x1.0p-53 * vmax;
		reinterpret_cast<long long*>(S)[2 * j] = key;
		reinterpret_cast<double*>(S)[2 * j + 1] = v;
	}
}

extern "C" int pg_generate_zipf_fk(pg_ctx* ctx, pg_stream stream, const void* R, uint64_t nR, double s,
		uint64_t seed, void* S, uint64_t nS, double vmax)
{
	if (!ctx || (nS && (!R || !S || nR == 0)) || s < 0.0) return pg_fail(ctx, PG_ERR_ARG, "pg_generate_zipf_fk: bad argument");
	if (nS == 0) return PG_OK;
	ZipfParams zp;
	zp.s = s; zp.n = nR;
	zp.hx1 = zf_H(s, 1.5) - 1.0;
	zp.hn = zf_H(s, (double) nR + 0.5);
	zp.sx = 2.0 - zf_Hinv(s, zf_H(s, 2.5) - zf_h(s, 2.0));
	const int blocks = (int) std::min<uint64_t>(pg_div_up(nS, 256), (uint64_t) ctx->sm_count * 16);
	k_generate_zipf_fk<<<blocks, 256, 0, (cudaStream_t) stream>>>((const char*) R, zp, seed, (char*) S, nS, vmax);
	PG_LAUNCHED(ctx);
	return PG_OK;
}
