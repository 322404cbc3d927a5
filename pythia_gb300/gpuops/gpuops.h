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
// Adjacent GPU operators exchange their data on the device. A GPU operator
// whose child is another GPU operator asks it, from init, to keep its output
// in device memory; each of its threads then takes its share of the child's
// output as a device span instead of reading pages, and the group's first
// thread runs its launch over the group's shares: in place when they are
// adjacent in the child's output, gathered by device copies otherwise. Only
// the leaves' pages cross to the device and only the top GPU operator's output
// comes back. This takes the place of the host-side page hand-over of
// MergeOp (operators/merge.cpp:433-543) between GPU operators.
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

// Data the operators moved (process-wide, bytes): pages uploaded to the
// device, outputs downloaded to pages, device copies gathering inputs, and
// the number of inputs taken on the device without any copy.
struct TransferStats {
	unsigned long long h2d, d2h, d2d, in_place;
	unsigned long long direct;   // of h2d: bytes copied straight from pinned or registered pages
};
TransferStats transfer_stats();
void reset_transfer_stats();
// Device exchange between adjacent GPU operators: on by default. Off, every
// operator reads and writes host pages (for comparison and tests); takes
// effect for operators initialised afterwards.
void set_device_exchange(bool on);

// Phase trace of the GPU operators, the counterpart of the engine's TRACELOG
// ring of (thread, label, timestamp) entries (operators/join.cpp:55-120):
// off by default; when on, operator threads append (plan node, thread,
// phase, host monotonic ns) entries to a fixed ring until it is full.
// trace_enable(true) also empties the ring; trace_dump writes one line per entry,
// "ns node thread phase", and returns the bytes the whole dump needs. Turn
// it on or off between plan runs, not while operator threads run.
void trace_enable(bool on);
void trace(const std::string& node, int tid, const char* phase);
unsigned long long trace_dump(char* buf, unsigned long long len);

// Rows of one operator thread's output in device memory.
struct DeviceSpan {
	const char* data;           // device pointer; NULL when rows == 0
	unsigned long long rows;
};

// A GPU operator that can leave its output on the device for a GPU parent.
class DeviceProducer {
public:
	DeviceProducer() : on_device_(false) { }
	virtual ~DeviceProducer() { }
	// Called by the parent's init: keep the output on the device; getNext
	// then reports Error (the parent takes device_share instead).
	virtual void keep_on_device() { on_device_ = true; }
	// After scanStart(tid) returned Ready: the rows thread `tid` serves,
	// valid until destroy.
	virtual DeviceSpan device_share(unsigned short tid) = 0;
protected:
	bool on_device_;
	std::string node_;          // plan node name, for the phase trace
};

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

// Per-group shared output and per-thread serving state. A group's output is
// either host memory served as pages, or device memory taken by a GPU parent.
class GroupedOutput {
public:
	GroupedOutput() : tuple_size_(0), page_bytes_(0) { pthread_mutex_init(&mu_, 0); }
	~GroupedOutput() { clear(); pthread_mutex_destroy(&mu_); }
	void setup(const ThreadGroups& g, unsigned tuple_size, unsigned buffsize);
	std::vector<char>& buffer(int group) { return out_[group]; }
	void set_rows(int group, unsigned long long rows) { rows_[group] = rows; }
	// The group's output is `rows` tuples at device address `data`.
	void set_device(int group, const char* data, unsigned long long rows);
	// Pool memory (pg_buffer_alloc_async) freed by clear(), after every
	// reader has synchronised; threads may hand it over concurrently.
	void own_device(void* p);
	// Thread `tid` serves rows [pos * rows / k, (pos + 1) * rows / k) of its group.
	void assign(int tid, int group, int pos, int k);
	Operator::GetNextResultT next(int tid);
	DeviceSpan share(int tid) const;
	void clear();
private:
	GroupedOutput(const GroupedOutput&);
	GroupedOutput& operator=(const GroupedOutput&);
	struct Cursor {
		char* at; unsigned long long left; Operator::Page* page; bool done;
		const char* dev; unsigned long long dev_rows;
	};
	pthread_mutex_t mu_;
	std::vector<std::vector<char> > out_;
	std::vector<unsigned long long> rows_;
	std::vector<const char*> dev_;
	std::vector<void*> owned_;
	std::vector<Cursor> cur_;
	unsigned tuple_size_, page_bytes_;
};

// Appends every tuple the child serves to `sink` until it reports Finished.
// Returns false when the child reports Error. (Inputs go through InputSide,
// which stages them for the device; this is its path without a GPU context.)
bool drain(Operator* child, unsigned short tid, std::vector<char>& sink);

// One input of a GPU operator. A host child's pages are staged on their way
// in: each thread copies the pages it reads into pinned buffers and sends
// every full buffer to device memory at once, so the upload overlaps the scan
// (operators/parallelscan.cpp:176-190 hands pages to its parent the same way,
// one page at a time). A GPU child keeping its output on the device gives
// each thread's device span instead.
class InputSide {
public:
	InputSide() : dev_(0) { }
	~InputSide() { clear(); }
	// From init: asks a GPU child to keep its output on the device; `node`
	// names the reading operator in the phase trace.
	void setup(Operator* child, const std::string& node);
	bool on_device() const { return dev_ != 0; }
	// After child->scanStart(tid): stages the pages or takes the span; false
	// when the child reported Error or the upload failed.
	bool fetch(Operator* child, unsigned short tid);
	// The rows of `members`, in order, as one device array of `width`-byte
	// tuples on stream `st`. *data points into the child's output or the
	// staged upload when that is one aligned run, else into *tmp (device
	// memory the caller frees after the stream's work).
	int gather(pg_ctx* ctx, pg_stream st, const std::vector<int>& members, unsigned width,
			const char** data, unsigned long long* rows, void** tmp);
	// The rows of `members` as the device arrays they lie in (GPU child spans
	// or staged chunks), in order, without copying: (data, tuples) pairs.
	// False when some rows are in host memory.
	bool pieces(const std::vector<int>& members, unsigned width,
			std::vector<std::pair<const char*, unsigned long long> >& out) const;
	// Frees thread `tid`'s staged input (after the work on `st` that reads it).
	void release(int tid, pg_stream st = 0);
	void clear();
private:
	InputSide(const InputSide&);
	InputSide& operator=(const InputSide&);
	struct Staged {
		std::vector<char*> chunks;                // device memory
		std::vector<unsigned long long> used;     // bytes of each chunk
	};
	bool stage(Operator* child, unsigned short tid);
	static bool flush(pg_ctx* ctx, pg_stream st, Staged& u, const char* buf, unsigned long long n,
			unsigned long long& room, unsigned long long& next_chunk, bool sm);
	DeviceProducer* dev_;
	std::vector<std::vector<char> > host_;        // pages read without a GPU context
	std::vector<Staged> staged_;
	std::vector<DeviceSpan> spans_;
	std::string node_;
};

class GpuFilterOp;

class GpuJoinBase : public DualInputOp, public DeviceProducer {
public:
	GpuJoinBase() : buildkey_(0), probekey_(0), probe_filter_(0) { }
	virtual void init(libconfig::Config& root, libconfig::Setting& node);
	virtual void threadInit(unsigned short threadid);
	virtual ResultCode scanStart(unsigned short threadid, Page* indexdatapage, Schema& indexdataschema);
	virtual GetNextResultT getNext(unsigned short threadid);
	virtual ResultCode scanStop(unsigned short threadid);
	virtual void threadClose(unsigned short threadid);
	virtual void destroy();
	virtual DeviceSpan device_share(unsigned short threadid) { return output_.share(threadid); }
	// A gpuproject above folds into the join, or a GPU join above reads only
	// some columns: output columns `keep` (indices into the current
	// projection), in that order.
	void narrow_projection(const std::vector<unsigned>& keep);
protected:
	// Whether run_device applies probe_preds_ itself (else the probe side is
	// filtered before it runs).
	virtual bool probe_predicates() const { return false; }
	// Joins device inputs on `st` into device rows *out (freed by the caller).
	virtual int run_device(pg_ctx* ctx, pg_stream st, const pg_rel& R, const pg_rel& S, void** out,
			unsigned long long* rows) = 0;
	// The same with the probe side as separate device arrays, not copied
	// together; PG_ERR_UNSUPPORTED sends the caller to run_device.
	virtual int run_device_spans(pg_ctx* ctx, pg_stream st, const pg_rel& R, const std::vector<pg_rel>& S,
			void** out, unsigned long long* rows)
	{
		(void) ctx; (void) st; (void) R; (void) S; (void) out; (void) rows;
		return PG_ERR_UNSUPPORTED;
	}
	std::vector<pg_col> cols_;
	unsigned buildkey_, probekey_;
	// Predicates of a gpufilter directly under the probe side, applied by
	// the join (the filter hands its input through).
	GpuFilterOp* probe_filter_;
	std::vector<pg_pred> probe_preds_;
private:
	int run_group(int g);
	ThreadGroups groups_;
	std::vector<GroupBarrier*> barriers_;
	InputSide build_, probe_;
	std::vector<int> group_rc_;
	GroupedOutput output_;
	pg_rel side_rel(Operator* child, unsigned attr, const void* data, unsigned long long rows);
};

// "gpuhashjoin": HashJoinOp's keys (operators/join.cpp:184-366): projection,
// buildjattr, probejattr, threadgroups; hash and tuplesperbucket are read and
// have no effect on the result.
class GpuHashJoinOp : public GpuJoinBase {
protected:
	virtual bool probe_predicates() const { return true; }
	virtual int run_device(pg_ctx* ctx, pg_stream st, const pg_rel& R, const pg_rel& S, void** out,
			unsigned long long* rows);
	virtual int run_device_spans(pg_ctx* ctx, pg_stream st, const pg_rel& R, const std::vector<pg_rel>& S,
			void** out, unsigned long long* rows);
};

// "gpumpsmjoin": OldMPSMJoinOp / MPSMJoinOp keys (join.cpp:677-783,
// 1383-1538): projection, buildjattr, probejattr, threadgroups, and
// buildpresorted / probepresorted = "yes" (join.cpp:750-762): the device
// confirms that the group's input on that side is sorted and then skips its
// sort or partition. maxbuildtuples[inM] / maxprobetuples[inM] size the CPU
// operator's staging runs, mostfreqbuildkeyoccurances its per-key buffer and
// buildprepartitioned the key range each CPU thread merges: device memory
// is sized from the inputs and any multiplicity is joined, so they are read
// and change nothing, the result included.
class GpuMPSMJoinOp : public GpuJoinBase {
public:
	GpuMPSMJoinOp() : sorted_flags_(0) { }
	virtual void init(libconfig::Config& root, libconfig::Setting& node);
protected:
	virtual int run_device(pg_ctx* ctx, pg_stream st, const pg_rel& R, const pg_rel& S, void** out,
			unsigned long long* rows);
private:
	int sorted_flags_;          // PG_JOIN_BUILD_SORTED / PG_JOIN_PROBE_SORTED
};

// "gpupartition": PartitionOp (operators/partition.cpp:45-404): `attr`,
// `range` and `buckets` (exactrange over [min, max] into `buckets`
// partitions, one per thread), or a `fn` other than exactrange with its
// options (parammodulo/knuth: skipbits, offset); `sort = "yes"` sorts each
// partition on `sortattr` (default `attr`). Thread t serves partition t.
// Tuples keep the order in which threads 0, 1, ... read them, as the
// reference's per-thread prefix sums arrange.
class GpuPartitionOp : public SingleInputOp, public DeviceProducer {
public:
	GpuPartitionOp() : attr_(0), sortattr_(0), sort_(false), nparts_(1) { }
	virtual DeviceSpan device_share(unsigned short threadid) { return served_.share(threadid); }
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
	int run_partition();
	GroupBarrier barrier_;
	InputSide in_;
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
class GpuAggregateOp : public SingleInputOp, public DeviceProducer {
public:
	explicit GpuAggregateOp(int agg) : agg_(agg), field_(-1), sumfield_(0), global_(false), threads_(1) { }
	virtual DeviceSpan device_share(unsigned short threadid) { return output_.share(threadid); }
	virtual void init(libconfig::Config& root, libconfig::Setting& node);
	virtual void threadInit(unsigned short threadid);
	virtual ResultCode scanStart(unsigned short threadid, Page* indexdatapage, Schema& indexdataschema);
	virtual GetNextResultT getNext(unsigned short threadid);
	virtual ResultCode scanStop(unsigned short threadid);
	virtual void destroy();
private:
	// Aggregates the shares of `members` into group `g` of the output.
	int aggregate(const std::vector<int>& members, int g);
	int agg_;
	int field_;
	unsigned sumfield_;
	bool global_;
	unsigned threads_;
	GroupBarrier barrier_;
	InputSide in_;
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

// "gpufilter": Filter (operators/filter.cpp:37-85): `field`, `op` ("<",
// "<=", "=", "==", "<>", "!=", ">=", ">") and `value`, text in the column's
// own form, parsed as Filter parses it (Schema::parseTuple). Each thread
// filters its own input, in order, as MapWrapper's per-thread loop does
// (mapwrapper.cpp:71-138). Fused forms: a gpufilter under another gpufilter
// hands its input up and the upper one evaluates both predicates in one
// launch; a gpufilter directly under the probe side of a gpuhashjoin hands
// its input to the join, whose probe evaluates the predicates before its
// table lookups (gpumpsmjoin filters the probe side on the device first).
class GpuFilterOp : public SingleInputOp, public DeviceProducer {
public:
	GpuFilterOp() : fused_(false) { }
	virtual void init(libconfig::Config& root, libconfig::Setting& node);
	virtual void threadInit(unsigned short threadid);
	virtual ResultCode scanStart(unsigned short threadid, Page* indexdatapage, Schema& indexdataschema);
	virtual GetNextResultT getNext(unsigned short threadid);
	virtual ResultCode scanStop(unsigned short threadid);
	virtual void destroy();
	virtual DeviceSpan device_share(unsigned short threadid) { return output_.share(threadid); }
	// Called by the parent that applies predicates() itself.
	void fuse_into_parent() { fused_ = true; keep_on_device(); }
	const std::vector<pg_pred>& predicates() const { return preds_; }
private:
	int run(unsigned short tid);
	std::vector<pg_pred> preds_;     // this filter's, then those of fused filters below
	bool fused_;
	InputSide in_;
	ThreadGroups groups_;            // one group per thread
	GroupedOutput output_;
	std::vector<int> rc_;
};

// "gpuproject": Project (operators/project.cpp:37-104): `projection` =
// ("$i", ...), the input columns to keep, in order. Over a GPU join it folds
// into the join's projection (the join writes only these columns) and hands
// the join's output through; otherwise each thread projects its own input.
class GpuProjectOp : public SingleInputOp, public DeviceProducer {
public:
	GpuProjectOp() : join_(0) { }
	virtual void init(libconfig::Config& root, libconfig::Setting& node);
	virtual void threadInit(unsigned short threadid);
	virtual ResultCode scanStart(unsigned short threadid, Page* indexdatapage, Schema& indexdataschema);
	virtual GetNextResultT getNext(unsigned short threadid);
	virtual ResultCode scanStop(unsigned short threadid);
	virtual void destroy();
	virtual DeviceSpan device_share(unsigned short threadid);
	virtual void keep_on_device();
private:
	int run(unsigned short tid);
	std::vector<unsigned> proj_;
	std::vector<pg_col> cols_;
	GpuJoinBase* join_;              // the join this projection folded into
	InputSide in_;
	ThreadGroups groups_;
	GroupedOutput output_;
	std::vector<int> rc_;
};

// The operator for a plan `type:` string ("gpuhashjoin", ...), or NULL.
Operator* create(const std::string& type);

}  // namespace pythia_gpu_ops

#endif
