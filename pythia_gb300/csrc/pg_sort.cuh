// Sorted-record interface shared by the page sort and the MPSM join.
#pragma once
#include "pg_internal.cuh"

struct __align__(16) pg_rec {
	long long key;            // sort key, widened to int64
	unsigned long long val;   // other half of a 16-byte tuple, or the row index
};

// 0: 16-byte tuple with its key at 0; 1: key at 8; 2: (key, row index) records.
int pg_sort_mode(const pg_rel* r);
int pg_sort_records(pg_ctx* ctx, cudaStream_t s, const pg_rel* in, pg_rec** recs);
