// Join-table images: a built table written to host memory (or a file) and
// loaded back onto a device without its build relation.
//
// Replaces HashTable::serialize / deserialize (util/hashtable.cpp:99-201) and
// the segment files they use (creatememsegment, operators/memsegmentwriter.cpp:
// 154-197; attachmemsegment, util/hashtable.cpp:124-178). The reference copies
// one partition's bucket memory byte for byte into a shared-memory segment and
// back into a table initialised with the same parameters. Here an image carries
// its own description, so a loader needs nothing but the bytes:
//
//   [header, 512 bytes][section 0][section 1]...[section 4]
//
// Sections start on 256-byte boundaries (zero padding between them): 0 hashed
// slots, 1 empty-marker side list, 2 dense values, 3 dense presence bits,
// 4 narrow dense entries; a layout leaves the sections it lacks empty. The
// header holds the layout, the key domain, the build projection and two
// checksums: one over the header itself and one over the payload, both
// sum_i w_i * (2 i + 1) mod 2^64 over 8-byte little-endian words w_i (i = the
// word's index in the image; a 4-byte tail counts as a zero-padded word). The
// payload checksum runs on the device, at HBM speed, after the copies.
//
// Only tables whose values are the packed build columns are self-contained;
// a table that stores build row indices (projected build columns wider than
// 8 bytes) refers to the build relation's memory and is refused.
#include "pg_internal.cuh"
#include "pg_hashtable.cuh"
#include <algorithm>
#include <cerrno>
#include <cstddef>
#include <cstring>
#include <fcntl.h>
#include <sys/stat.h>
#include <unistd.h>

#define IMG_MAGIC "PGJTABLE"
#define IMG_VERSION 1u
#define IMG_HEADER 512u
#define IMG_SECTIONS 5
#define IMG_ALIGN 256u

enum { IMG_HASHED = 0, IMG_DENSE = 1, IMG_DENSE32 = 2 };

struct ImgHeader {
	char magic[8];
	uint32_t version;
	uint32_t header_bytes;
	uint32_t layout;
	uint32_t flags;             // bit 0: unique keys
	uint64_t nbuild;
	uint32_t wR, bkey_bytes;
	uint32_t log2cap, nside;
	int64_t dmin;
	uint64_t drange;
	uint64_t vmin, vmax;
	uint32_t nproj, reserved;
	pg_col proj[HJ_MAX_COLS];
	uint64_t sec_off[IMG_SECTIONS];
	uint64_t sec_bytes[IMG_SECTIONS];
	uint64_t image_bytes;
	uint64_t payload_sum;
	uint8_t pad[IMG_HEADER - 8 - 4 * 4 - 8 - 4 * 4 - 8 * 4 - 4 * 2 - 12 * HJ_MAX_COLS
			- 16 * IMG_SECTIONS - 8 * 3];
	uint64_t header_sum;        // over every word before this one
};
static_assert(sizeof(ImgHeader) == IMG_HEADER, "image header is 512 bytes");

// Weighted word sum of `nbytes` bytes at `p`, whose first word is word
// `base` of the image. Device pointers from the pool are 256-byte aligned.
__global__ void k_image_sum(const unsigned long long* __restrict__ p, uint64_t nbytes, uint64_t base,
		unsigned long long* __restrict__ acc)
{
	const uint64_t nw = nbytes / 8;
	unsigned long long s = 0;
	const uint64_t stride = (uint64_t) gridDim.x * blockDim.x;
	for (uint64_t i = (uint64_t) blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += stride)
		s += __ldcs(p + i) * (2 * (base + i) + 1);
	if (blockIdx.x == 0 && threadIdx.x == 0 && (nbytes & 7)) {
		// 4-byte tail (sections are whole 4-byte words): zero-padded word.
		const unsigned long long t = reinterpret_cast<const uint32_t*>(p + nw)[0];
		s += t * (2 * (base + nw) + 1);
	}
	for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
	if ((threadIdx.x & 31) == 0 && s) atomicAdd(acc, s);
}

static uint64_t host_sum(const void* p, uint64_t nbytes, uint64_t base)
{
	const unsigned char* b = (const unsigned char*) p;
	uint64_t s = 0;
	for (uint64_t i = 0; i * 8 < nbytes; ++i) {
		uint64_t w = 0;
		memcpy(&w, b + i * 8, std::min<uint64_t>(8, nbytes - i * 8));
		s += w * (2 * (base + i) + 1);
	}
	return s;
}

static uint64_t img_align(uint64_t x) { return (x + IMG_ALIGN - 1) / IMG_ALIGN * IMG_ALIGN; }

// Section sizes for the layout fields of `h`; offsets and image size follow.
static void img_layout(ImgHeader& h)
{
	for (int i = 0; i < IMG_SECTIONS; ++i) h.sec_bytes[i] = 0;
	if (h.layout == IMG_HASHED) {
		h.sec_bytes[0] = 16ull << h.log2cap;
		h.sec_bytes[1] = 8ull * h.nside;
	} else if (h.layout == IMG_DENSE) {
		h.sec_bytes[2] = 8 * h.drange;
		h.sec_bytes[3] = 4 * pg_div_up(h.drange, 32);
	} else {
		h.sec_bytes[4] = 4 * h.drange;
	}
	uint64_t off = IMG_HEADER;
	for (int i = 0; i < IMG_SECTIONS; ++i) {
		h.sec_off[i] = h.sec_bytes[i] ? off : 0;
		off = img_align(off + h.sec_bytes[i]);
	}
	h.image_bytes = off;
}

static int table_header(pg_ctx* ctx, const pg_hashtable* ht, ImgHeader& h)
{
	// An image describes the exact layout: a table still checked on the
	// device is settled first (the table is logically unchanged).
	if (int rc = hj_settle(ctx, const_cast<pg_hashtable*>(ht))) return rc;
	if (!ht->inline_val)
		return pg_fail(ctx, PG_ERR_UNSUPPORTED,
				"table image: the table stores build row indices (build columns wider than 8 bytes)");
	memset(&h, 0, sizeof(h));
	memcpy(h.magic, IMG_MAGIC, 8);
	h.version = IMG_VERSION;
	h.header_bytes = IMG_HEADER;
	h.layout = ht->dense32 ? IMG_DENSE32 : ht->dense ? IMG_DENSE : IMG_HASHED;
	h.flags = ht->unique ? 1 : 0;
	h.nbuild = ht->nbuild;
	h.wR = ht->wR; h.bkey_bytes = ht->bkey_bytes;
	h.log2cap = ht->dense ? 0 : ht->log2cap;
	h.nside = ht->dense ? 0 : ht->nside;
	h.dmin = ht->dense ? ht->dmin : 0;
	h.drange = ht->dense ? ht->drange : 0;
	h.vmin = ht->vmin; h.vmax = ht->vmax;
	h.nproj = (uint32_t) ht->nproj;
	for (int i = 0; i < ht->nproj; ++i) h.proj[i] = ht->proj[i];
	img_layout(h);
	return PG_OK;
}

static int launch_sum(pg_ctx* ctx, cudaStream_t s, const void* p, uint64_t nbytes, uint64_t off,
		unsigned long long* acc)
{
	if (!nbytes) return PG_OK;
	const int blocks = (int) std::max<uint64_t>(1, std::min<uint64_t>(pg_div_up(nbytes / 8, 256 * 8),
			(uint64_t) ctx->sm_count * 8));
	k_image_sum<<<blocks, 256, 0, s>>>((const unsigned long long*) p, nbytes, off / 8, acc);
	PG_LAUNCHED(ctx);
	return PG_OK;
}

static const void* table_section(const pg_hashtable* ht, int i)
{
	switch (i) {
	case 0: return ht->slots;
	case 1: return ht->side;
	case 2: return ht->dense_val;
	case 3: return ht->dense_bits;
	default: return ht->dense32;
	}
}

extern "C" int pg_hashtable_image_size(pg_ctx* ctx, const pg_hashtable* ht, uint64_t* bytes)
{
	if (!ctx || !ht || !bytes) return pg_fail(ctx, PG_ERR_ARG, "pg_hashtable_image_size: null argument");
	ImgHeader h;
	int rc;
	if ((rc = table_header(ctx, ht, h))) return rc;
	*bytes = h.image_bytes;
	return PG_OK;
}

extern "C" int pg_hashtable_serialize(pg_ctx* ctx, pg_stream stream, const pg_hashtable* ht,
		void* image, uint64_t capacity, uint64_t* bytes)
{
	if (!ctx || !ht || !bytes) return pg_fail(ctx, PG_ERR_ARG, "pg_hashtable_serialize: null argument");
	ImgHeader h;
	int rc;
	if ((rc = table_header(ctx, ht, h))) return rc;
	*bytes = h.image_bytes;
	if (!image) return PG_OK;
	if (capacity < h.image_bytes)
		return pg_fail(ctx, PG_ERR_OUTPUT_FULL, "pg_hashtable_serialize: image buffer too small");
	cudaStream_t s = (cudaStream_t) stream;
	unsigned long long* acc = nullptr;
	if ((rc = pg_alloc_async(ctx, s, (void**) &acc, 64))) return rc;
	PG_CUDA(ctx, cudaMemsetAsync(acc, 0, 8, s));
	char* img = (char*) image;
	uint64_t prev_end = IMG_HEADER;
	for (int i = 0; i < IMG_SECTIONS; ++i)
		if (h.sec_bytes[i] && (reinterpret_cast<uintptr_t>(table_section(ht, i)) & 15))
			return pg_fail(ctx, PG_ERR_ARG, "pg_hashtable_serialize: table array not 16-byte aligned");
	for (int i = 0; i < IMG_SECTIONS; ++i) {
		if (!h.sec_bytes[i]) continue;
		memset(img + prev_end, 0, h.sec_off[i] - prev_end);
		if ((rc = launch_sum(ctx, s, table_section(ht, i), h.sec_bytes[i], h.sec_off[i], acc))) return rc;
		PG_CUDA(ctx, cudaMemcpyAsync(img + h.sec_off[i], table_section(ht, i), h.sec_bytes[i],
				cudaMemcpyDeviceToHost, s));
		prev_end = h.sec_off[i] + h.sec_bytes[i];
	}
	memset(img + prev_end, 0, h.image_bytes - prev_end);
	unsigned long long sum = 0;
	PG_CUDA(ctx, cudaMemcpyAsync(&sum, acc, 8, cudaMemcpyDeviceToHost, s));
	pg_free_async(ctx, s, acc);
	PG_CUDA(ctx, cudaStreamSynchronize(s));
	h.payload_sum = sum;
	h.header_sum = host_sum(&h, offsetof(ImgHeader, header_sum), 0);
	memcpy(img, &h, sizeof(h));
	return PG_OK;
}

static int img_bad(pg_ctx* ctx, const char* what)
{
	return pg_fail(ctx, PG_ERR_ARG, std::string("pg_hashtable_deserialize: ") + what);
}

// Checks an image header against the image's size; fills `h`.
static int img_check(pg_ctx* ctx, const void* image, uint64_t bytes, ImgHeader& h)
{
	if (bytes < IMG_HEADER) return img_bad(ctx, "image shorter than its header");
	memcpy(&h, image, sizeof(h));
	if (memcmp(h.magic, IMG_MAGIC, 8)) return img_bad(ctx, "not a join-table image");
	if (h.version != IMG_VERSION || h.header_bytes != IMG_HEADER) return img_bad(ctx, "unknown image version");
	if (h.header_sum != host_sum(&h, offsetof(ImgHeader, header_sum), 0)) return img_bad(ctx, "header checksum mismatch");
	if (h.layout > IMG_DENSE32 || h.nproj > HJ_MAX_COLS) return img_bad(ctx, "bad layout");
	if (h.layout == IMG_HASHED ? (h.log2cap < 1 || h.log2cap > 40 || h.drange)
			: (h.drange == 0 || h.drange >= (1ull << 34) || h.log2cap || h.nside))
		return img_bad(ctx, "bad key domain");
	if (h.layout == IMG_HASHED && h.nside > h.nbuild) return img_bad(ctx, "bad side list");
	uint32_t bbytes = 0;
	for (uint32_t i = 0; i < h.nproj; ++i) {
		const pg_col& c = h.proj[i];
		if (c.side > 1 || (c.bytes != 4 && c.bytes != 8) || (c.off & 3) || (c.side == 0 && c.off + c.bytes > h.wR))
			return img_bad(ctx, "bad projection");
		if (c.side == 0) bbytes += c.bytes;
	}
	if (bbytes > 8) return img_bad(ctx, "bad projection");
	ImgHeader want = h;
	img_layout(want);
	for (int i = 0; i < IMG_SECTIONS; ++i)
		if (want.sec_off[i] != h.sec_off[i] || want.sec_bytes[i] != h.sec_bytes[i])
			return img_bad(ctx, "section table does not match the layout");
	if (want.image_bytes != h.image_bytes) return img_bad(ctx, "image size does not match the layout");
	if (bytes < h.image_bytes) return img_bad(ctx, "image truncated");
	return PG_OK;
}

extern "C" int pg_hashtable_deserialize(pg_ctx* ctx, pg_stream stream, const void* image, uint64_t bytes,
		pg_hashtable** out)
{
	if (!ctx || !image || !out) return pg_fail(ctx, PG_ERR_ARG, "pg_hashtable_deserialize: null argument");
	*out = nullptr;
	ImgHeader h;
	int rc;
	if ((rc = img_check(ctx, image, bytes, h))) return rc;
	cudaStream_t s = (cudaStream_t) stream;
	pg_hashtable* ht = new pg_hashtable();
	ht->nbuild = h.nbuild; ht->R = nullptr; ht->wR = h.wR; ht->bkey_bytes = h.bkey_bytes;
	ht->nproj = (int) h.nproj;
	ht->stream = s;
	ht->bcols.n = 0;
	for (uint32_t i = 0; i < h.nproj; ++i) {
		ht->proj[i] = h.proj[i];
		if (h.proj[i].side == 0) {
			ht->bcols.roff[ht->bcols.n] = (uint16_t) (h.proj[i].off / 4);
			ht->bcols.words[ht->bcols.n] = (uint8_t) (h.proj[i].bytes / 4);
			ht->bcols.n++;
		}
	}
	ht->inline_val = true;
	ht->unique = (h.flags & 1) != 0;
	ht->dense = h.layout != IMG_HASHED;
	ht->dmin = h.dmin; ht->drange = h.drange; ht->vmin = h.vmin; ht->vmax = h.vmax; ht->vlo = h.vmin;
	ht->log2cap = ht->dense ? 1 : h.log2cap;
	ht->capacity = ht->dense ? 0 : 1ull << h.log2cap;
	ht->nside = h.nside;
	ht->side_cap = h.nside;
	void** dst[IMG_SECTIONS] = {(void**) &ht->slots, (void**) &ht->side, (void**) &ht->dense_val,
		(void**) &ht->dense_bits, (void**) &ht->dense32};
	unsigned long long* acc = nullptr;
	for (int i = 0; i < IMG_SECTIONS; ++i) {
		// The hashed layout always has a side list (possibly empty).
		const uint64_t nb = h.sec_bytes[i] ? h.sec_bytes[i] : (i == 1 && !ht->dense ? 64 : 0);
		if (nb && (rc = pg_alloc_async(ctx, s, dst[i], nb))) { pg_hashtable_free(ctx, ht); return rc; }
	}
	if ((rc = pg_alloc_async(ctx, s, (void**) &acc, 64))) { pg_hashtable_free(ctx, ht); return rc; }
	unsigned long long sum = 0;
	cudaError_t e = cudaMemsetAsync(acc, 0, 8, s);
	for (int i = 0; i < IMG_SECTIONS && e == cudaSuccess; ++i) {
		if (!h.sec_bytes[i]) continue;
		e = cudaMemcpyAsync(*dst[i], (const char*) image + h.sec_off[i], h.sec_bytes[i], cudaMemcpyHostToDevice, s);
		if (e == cudaSuccess && (rc = launch_sum(ctx, s, *dst[i], h.sec_bytes[i], h.sec_off[i], acc))) {
			pg_free_async(ctx, s, acc); pg_hashtable_free(ctx, ht); return rc;
		}
	}
	if (e == cudaSuccess) e = cudaMemcpyAsync(&sum, acc, 8, cudaMemcpyDeviceToHost, s);
	pg_free_async(ctx, s, acc);
	if (e == cudaSuccess) e = cudaStreamSynchronize(s);
	if (e != cudaSuccess) { pg_hashtable_free(ctx, ht); return pg_cuda_fail(ctx, e, "pg_hashtable_deserialize"); }
	// Padding between sections is zero in a well-formed image; a section's
	// words and their positions are what the sum covers.
	if (sum != h.payload_sum) { pg_hashtable_free(ctx, ht); return img_bad(ctx, "payload checksum mismatch"); }
	*out = ht;
	return PG_OK;
}

static int io_fail(pg_ctx* ctx, const char* what, const char* path)
{
	return pg_fail(ctx, PG_ERR_ARG, std::string(what) + ": " + path + ": " + strerror(errno));
}

extern "C" int pg_hashtable_save(pg_ctx* ctx, pg_stream stream, const pg_hashtable* ht, const char* path)
{
	if (!ctx || !ht || !path) return pg_fail(ctx, PG_ERR_ARG, "pg_hashtable_save: null argument");
	uint64_t n = 0;
	int rc;
	if ((rc = pg_hashtable_image_size(ctx, ht, &n))) return rc;
	void* img = nullptr;
	PG_CUDA(ctx, cudaMallocHost(&img, n));
	if ((rc = pg_hashtable_serialize(ctx, stream, ht, img, n, &n))) { cudaFreeHost(img); return rc; }
	// A new file only, as the reference's segment writer creates them.
	const int fd = open(path, O_WRONLY | O_CREAT | O_EXCL, 0600);
	if (fd < 0) { cudaFreeHost(img); return io_fail(ctx, "pg_hashtable_save: cannot create", path); }
	uint64_t done = 0;
	while (done < n) {
		const ssize_t w = write(fd, (const char*) img + done, (size_t) std::min<uint64_t>(n - done, 1ull << 30));
		if (w < 0 && errno == EINTR) continue;
		if (w <= 0) { rc = io_fail(ctx, "pg_hashtable_save: write failed", path); break; }
		done += (uint64_t) w;
	}
	if (close(fd) != 0 && !rc) rc = io_fail(ctx, "pg_hashtable_save: close failed", path);
	cudaFreeHost(img);
	if (rc) unlink(path);
	return rc;
}

extern "C" int pg_hashtable_load(pg_ctx* ctx, pg_stream stream, const char* path, pg_hashtable** out)
{
	if (!ctx || !path || !out) return pg_fail(ctx, PG_ERR_ARG, "pg_hashtable_load: null argument");
	*out = nullptr;
	const int fd = open(path, O_RDONLY);
	if (fd < 0) return io_fail(ctx, "pg_hashtable_load: cannot open", path);
	struct stat st;
	if (fstat(fd, &st) != 0) { close(fd); return io_fail(ctx, "pg_hashtable_load: cannot stat", path); }
	const uint64_t n = (uint64_t) st.st_size;
	void* img = nullptr;
	cudaError_t e = cudaMallocHost(&img, n ? n : 16);
	if (e != cudaSuccess) { close(fd); return pg_cuda_fail(ctx, e, "cudaMallocHost"); }
	uint64_t done = 0;
	int rc = PG_OK;
	while (done < n) {
		const ssize_t r = read(fd, (char*) img + done, (size_t) std::min<uint64_t>(n - done, 1ull << 30));
		if (r < 0 && errno == EINTR) continue;
		if (r <= 0) { rc = io_fail(ctx, "pg_hashtable_load: read failed", path); break; }
		done += (uint64_t) r;
	}
	close(fd);
	if (!rc) rc = pg_hashtable_deserialize(ctx, stream, img, n, out);
	cudaFreeHost(img);
	return rc;
}
