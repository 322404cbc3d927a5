// GPU operators for Pythia plans: gpuhashjoin, gpumpsmjoin, gpupartition,
// gpuaggregate_sum, gpuaggregate_count. Each class is a Pythia operator
// (DualInputOp or SingleInputOp) that keeps its CPU counterpart's plan keys,
// output schema and per-thread page contract, and runs the work through the
// C ABI of libpythia_gpu (include/pythia_gpu.h):
//
//   init         parses the same keys as the CPU operator and fills `schema`;
//   scanStart    drains this thread's input pages into host memory, meets the
//                other threads of its group at a barrier, the group's first
//                thread runs the GPU operator once over the group's input
//                (threads' inputs concatenated in group order), and all meet
//                again; a GPU failure makes every thread of the group return
//                Error;
//   getNext      serves this thread's share of the group's output as
//                zero-copy pages of at most `buffsize` bytes; the last page
//                comes with Finished, and Finished repeats after that;
//   scanStop     propagates down;
//   destroy      frees the outputs.
//
// Compiled against the engine's own headers (PYTHIA_REFERENCE_HEADERS) the
// classes drop into its plans; otherwise against the mirror of its operator
// interface in mirror/pythia_mirror.h.
#ifndef PYTHIA_GPUOPS_H
#define PYTHIA_GPUOPS_H

#ifdef PYTHIA_REFERENCE_HEADERS
#include "operators/operators.h"
#else
#include "mirror/pythia_mirror.h"
#endif

#include <pthread.h>
#include <string>
#include <vector>

#include "pythia_gpu.h"

namespace pythia_gpu_ops {

// Process-wide GPU context (device 0), made on first use. NULL when no GPU
// or the library failed to start; the operators then return Error.
pg_ctx* shared_context();
// Message of the last failure seen by an operator of this process.
std::string last_failure();

class GroupBarrier {
public:
	GroupBarrier() : size_(1), waiting_(0), phase_(0)
	{
		pthread_mutex_init(&mu_, 0);
		pthread_cond_init(&cv_, 0);
	}
	~GroupBarrier() { pthread_mutex_destroy(&mu_); pthread_cond_destroy(&cv_); }
	void init(unsigned n) { size_ = n ? n : 1; }
	void arrive();
private:
	GroupBarrier(const GroupBarrier&);
	GroupBarrier& operator=(const GroupBarrier&);
	pthread_mutex_t mu_;
	pthread_cond_t cv_;
	unsigned size_, waiting_, phase_;
};

// Thread groups as HashJoinOp reads them (`threadgroups = ((0, 1), (2, 3))`,
// operators/join.cpp:203-238), or one group of `threads` threads.
struct ThreadGroups {
	std::vector<int> group_of, pos_in;          // by thread id
	std::vector<std::vector<int> > members;     // by group
	void parse(libconfig::Setting& node, int default_threads);
};

// Per-group shared output and per-thread serving state.
class GroupedOutput {
public:
	GroupedOutput() : tuple_size_(0), page_bytes_(0) { }
	~GroupedOutput() { clear(); }
	void setup(const ThreadGroups& g, unsigned tuple_size, unsigned buffsize);
	std::vector<char>& buffer(int group) { return out_[group]; }
	void set_rows(int group, unsigned long long rows) { rows_[group] = rows; }
	// Thread `tid` serves rows [pos * rows / k, (pos + 1) * rows / k) of its group.
	void assign(int tid, int group, int pos, int k);
	Operator::GetNextResultT next(int tid);
	void clear();
private:
	struct Cursor { char* at; unsigned long long left; Operator::Page* page; bool done; };
	std::vector<std::vector<char> > out_;
	std::vector<unsigned long long> rows_;
	std::vector<Cursor> cur_;
	unsigned tuple_size_, page_bytes_;
};

// Appends every tuple the child serves to `sink` until it reports Finished.
// Returns false when the child reports Error.
bool drain(Operator* child, unsigned short tid, std::vector<char>& sink);

class GpuJoinBase : public DualInputOp {
public:
	GpuJoinBase() : buildkey_(0), probekey_(0) { }
	virtual void init(libconfig::Config& root, libconfig::Setting& node);
	virtual void threadInit(unsigned short threadid);
	virtual ResultCode scanStart(unsigned short threadid, Page* indexdatapage, Schema& indexdataschema);
	virtual GetNextResultT getNext(unsigned short threadid);
	virtual ResultCode scanStop(unsigned short threadid);
	virtual void threadClose(unsigned short threadid);
	virtual void destroy();
protected:
	// Runs the join of one group's inputs into `out`; returns a PG_* code.
	virtual int run_group(const pg_rel& R, const pg_rel& S, std::vector<char>& out,
			unsigned long long* rows) = 0;
	std::vector<pg_col> cols_;
	unsigned buildkey_, probekey_;
private:
	ThreadGroups groups_;
	std::vector<GroupBarrier*> barriers_;
	std::vector<std::vector<char> > build_in_, probe_in_;
	std::vector<int> group_rc_;
	GroupedOutput output_;
	pg_rel side_rel(Operator* child, unsigned attr, const std::vector<char>& data);
};

// "gpuhashjoin": HashJoinOp's keys (operators/join.cpp:184-366): projection,
// buildjattr, probejattr, threadgroups; hash and tuplesperbucket are read and
// have no effect on the result.
class GpuHashJoinOp : public GpuJoinBase {
protected:
	virtual int run_group(const pg_rel& R, const pg_rel& S, std::vector<char>& out, unsigned long long* rows);
};

// "gpumpsmjoin": OldMPSMJoinOp / MPSMJoinOp keys (join.cpp:677-783,
// 1383-1538): projection, buildjattr, probejattr, threadgroups; the run-size
// and presorted keys are read and have no effect on the result.
class GpuMPSMJoinOp : public GpuJoinBase {
protected:
	virtual int run_group(const pg_rel& R, const pg_rel& S, std::vector<char>& out, unsigned long long* rows);
};

// "gpupartition": PartitionOp (operators/partition.cpp:45-404): `attr`,
// `range` and `buckets` (exactrange over [min, max] into `buckets`
// partitions, one per thread), or a `fn` other than exactrange with its
// options (parammodulo/knuth: skipbits, offset); `sort = "yes"` sorts each
// partition on `sortattr` (default `attr`). Thread t serves partition t.
// Tuples keep the order in which threads 0, 1, ... read them, as the
// reference's per-thread prefix sums arrange.
class GpuPartitionOp : public SingleInputOp {
public:
	GpuPartitionOp() : attr_(0), sortattr_(0), sort_(false), nparts_(1) { }
	virtual void init(libconfig::Config& root, libconfig::Setting& node);
	virtual void threadInit(unsigned short threadid);
	virtual ResultCode scanStart(unsigned short threadid, Page* indexdatapage, Schema& indexdataschema);
	virtual GetNextResultT getNext(unsigned short threadid);
	virtual ResultCode scanStop(unsigned short threadid);
	virtual void destroy();
private:
	unsigned attr_, sortattr_;
	bool sort_;
	unsigned nparts_;
	pg_hashcfg cfg_;
	GroupBarrier barrier_;
	std::vector<std::vector<char> > in_;
	std::vector<char> out_;
	std::vector<uint64_t> offsets_;
	int rc_;
	ThreadGroups one_group_;
	GroupedOutput served_;
};

// "gpuaggregate_sum" / "gpuaggregate_count": GenericAggregate with
// AggregateSum / AggregateCount (genericaggregate.cpp:51-487,
// aggregatesum.cpp:37-107, aggregatecount.cpp:37-52). `field` (one group-by
// column of 4 or 8 bytes) or `fields` (empty: one global group); `sumfield`
// for the sum; `global` with `threads` aggregates all threads' input once and
// spreads the groups over the threads, otherwise every thread aggregates and
// emits its own input. Output: (group column, aggregate), the aggregate typed
// like the summed column (sum) or long (count).
class GpuAggregateOp : public SingleInputOp {
public:
	explicit GpuAggregateOp(int agg) : agg_(agg), field_(-1), sumfield_(0), global_(false), threads_(1) { }
	virtual void init(libconfig::Config& root, libconfig::Setting& node);
	virtual void threadInit(unsigned short threadid);
	virtual ResultCode scanStart(unsigned short threadid, Page* indexdatapage, Schema& indexdataschema);
	virtual GetNextResultT getNext(unsigned short threadid);
	virtual ResultCode scanStop(unsigned short threadid);
	virtual void destroy();
private:
	int aggregate(const std::vector<char>& in, std::vector<char>& out, unsigned long long* groups);
	int agg_;
	int field_;
	unsigned sumfield_;
	bool global_;
	unsigned threads_;
	GroupBarrier barrier_;
	std::vector<std::vector<char> > in_;
	int rc_;
	ThreadGroups groups_;
	GroupedOutput output_;
};

class GpuAggregateSumOp : public GpuAggregateOp {
public:
	GpuAggregateSumOp() : GpuAggregateOp(PG_AGG_SUM) { }
};

class GpuAggregateCountOp : public GpuAggregateOp {
public:
	GpuAggregateCountOp() : GpuAggregateOp(PG_AGG_COUNT) { }
};

// The operator for a plan `type:` string ("gpuhashjoin", ...), or NULL.
Operator* create(const std::string& type);

}  // namespace pythia_gpu_ops

#endif
