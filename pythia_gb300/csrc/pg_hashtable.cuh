// Device-resident join table shared by the build, the probes and the table
// image (serialise / deserialise) code.
#ifndef PG_HASHTABLE_CUH
#define PG_HASHTABLE_CUH

#include "pg_internal.cuh"

#define HJ_MAX_COLS 16

struct HjBuildCols {            // build-projected columns packed into the value
	int n;
	uint16_t roff[HJ_MAX_COLS]; // word offset in the build tuple
	uint8_t words[HJ_MAX_COLS];
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
};

#endif
