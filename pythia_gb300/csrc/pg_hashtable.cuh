// Device-resident join table shared by the build, the probes and the table
// image (serialise / deserialise) code.
#ifndef PG_HASHTABLE_CUH
#define PG_HASHTABLE_CUH

#include "pg_internal.cuh"
#include <atomic>
#include <mutex>

#define HJ_MAX_COLS 16

struct HjBuildCols {            // build-projected columns packed into the value
	int n;
	uint16_t roff[HJ_MAX_COLS]; // word offset in the build tuple
	uint8_t words[HJ_MAX_COLS];
};

// Narrow dense table built without host round trips: a sample of the build
// side sets the key window and the value base on the device, the fill, store
// and count kernels read them here, and the store and count kernels record
// what the table must satisfy. A table whose header says "bad" is rebuilt
// exactly on its first use (hj_settle).
struct HjDenseHdr {
	long long dmin;              // key of entry 0 (window base)
	unsigned long long drange;   // window entries (0 when the sample ruled the layout out)
	unsigned long long vmin;     // entry = packed value - vmin
	unsigned long long n;        // build tuples
	unsigned long long present;  // entries the count pass found written
	unsigned long long kmin, kmax;   // exact key range (keys ^ 2^63, as unsigned), store pass
	unsigned long long vlo, vhi;     // exact packed-value range, store pass
	int flags;                   // 1 key outside the window, 2 value outside the entry range,
	                             // 4 sample: window larger than the allocation or values too wide
	int pad;
};

struct pg_hashtable {
	unsigned long long* slots;  // 2 * capacity words
	uint64_t capacity;
	uint32_t log2cap;
	uint64_t nbuild;
	bool unique;
	bool inline_val;            // value = packed build columns, else row index
	HjBuildCols bcols;
	const char* R;              // build tuples (row-index mode gathers from here)
	uint32_t wR;
	uint32_t bkey_bytes;
	unsigned long long* side;   // values of build tuples whose key is the empty marker
	uint32_t side_cap;
	uint32_t nside;
	pg_col proj[HJ_MAX_COLS];
	int nproj;
	cudaStream_t stream;        // stream the table was built on
	// Dense layout (unique keys spanning at most twice |R| values): value and
	// presence bit indexed by key - dmin instead of hashed slots.
	bool dense;
	unsigned long long* dense_val;
	uint32_t* dense_bits;
	long long dmin;
	unsigned long long drange;
	// Narrow dense layout: 4-byte entries holding value - vmin (frame of
	// reference), all ones for an absent key; used when the packed build
	// values span fewer than 2^32 - 1 values. Halves the table (a 16M-key
	// table is 64 MB, which stays in L2) and needs no presence bitmap.
	uint32_t* dense32;
	unsigned long long vmin;
	unsigned long long vmax;    // largest packed value (dense tables)
	unsigned long long vlo;     // smallest packed value (dense tables; vmin is the entries' base)
	// Speculative narrow dense table (built on the device, not yet checked
	// by the host). While `spec` holds, only dense32_base and hdr (the window
	// and the checks) describe the table; both stay allocated until the
	// table is freed, so kernels queued from other threads stay valid while
	// one thread settles it. Settling narrows the host-side fields (dense32 =
	// dense32_base + offset), writes a re-based copy of the entries when the
	// sample's value base is not the smallest value (dense32_copy), or
	// rebuilds a refuted table; it never rewrites the window's entries.
	std::atomic<bool> spec;
	std::mutex mu;              // serialises settling
	HjDenseHdr* hdr;
	uint32_t* dense32_base;
	uint32_t* dense32_copy;
	cudaEvent_t built;          // recorded after the speculative build's kernels (null otherwise)
	pg_rel rel;                 // the build relation, for an exact rebuild
};

// Makes a speculative table exact before a use that needs host-side layout
// facts: reads its header (one synchronisation of the build stream), narrows
// the window to the exact key range and, when the checks failed, rebuilds the
// table from the build relation. A no-op for other tables.
int hj_settle(pg_ctx* ctx, pg_hashtable* ht);

#endif
