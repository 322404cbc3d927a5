// Plan factory of the engine with the GPU operators registered.
//
// The engine turns a libconfig plan into an operator tree in Query::create
// (query.cpp:62-252): every node's `type` picks an operator class from a fixed
// list, the joins (dual-input types) among them, and only single-input types
// can be added from outside (Query::UserDefinedOpMapT, query.h:106). This file
// replaces the engine's query.o: it defines Query::create and
// Query::getOperatorDepth, with the engine's type names (the scans, joins and
// single-input operators of a build without HDF5 or FastBit) and the GPU
// operators' (gpuhashjoin, gpumpsmjoin, gpupartition, gpuaggregate_sum,
// gpuaggregate_count, gpufilter, gpuproject). A tree is built as the engine
// builds it: a node's operator is created, then its children's subtrees, then
// the node's init with its children already initialised; user-defined
// operators are claimed from the map (its entry is cleared). Linked before the
// engine's archive, so that query.o is not pulled from it:
//
//   g++ ... query_factory.o gpuops_ref.o libpythiaref.a -lpythia_gpu
//
// Compiled only against the engine's own headers (PYTHIA_REFERENCE_HEADERS).
#include <cstring>
#include <string>

#include "libconfig.h++"
#include "query.h"
#include "exceptions.h"
#include "operators/operators.h"

#include "gpuops.h"

namespace {

// Operator constructors by the number of inputs they take.
typedef ZeroInputOp* (*MakeScan)();
typedef SingleInputOp* (*MakeSingle)();
typedef DualInputOp* (*MakeDual)();

template <class T> ZeroInputOp* scan() { return new T(); }
template <class T> SingleInputOp* single() { return new T(); }
template <class T> DualInputOp* dual() { return new T(); }

struct ScanKind { const char* type; MakeScan make; };
struct SingleKind { const char* type; MakeSingle make; };
struct DualKind { const char* type; MakeDual make; };

const ScanKind scans[] = {
	{"scan", scan<ScanOp>},
	{"partitionedscan", scan<PartitionedScanOp>},
	{"parallelscan", scan<ParallelScanOp>},
	{"generator_int", scan<IntGeneratorOp>},
};

// Children: "build" (buildOp) and "probe" (probeOp).
const DualKind duals[] = {
	{"hashjoin", dual<HashJoinOp>},
	{"sortmergejoin", dual<SortMergeJoinOp>},
	{"mpsmjoin", dual<OldMPSMJoinOp>},
	{"newmpsmjoin", dual<MPSMJoinOp>},
	{"preprejoin", dual<PresortedPrepartitionedMergeJoinOp>},
	{"indexhashjoin", dual<IndexHashJoinOp>},
	{"gpuhashjoin", dual<pythia_gpu_ops::GpuHashJoinOp>},
	{"gpumpsmjoin", dual<pythia_gpu_ops::GpuMPSMJoinOp>},
};

// Child: "input" (nextOp).
const SingleKind singles[] = {
	{"aggregate_sum", single<AggregateSum>},
	{"aggregate_count", single<AggregateCount>},
	{"merge", single<MergeOp>},
	{"shmwriter", single<MemSegmentWriter>},
	{"filter", single<Filter>},
	{"cycle_accountant", single<CycleAccountant>},
	{"projection", single<Project>},
	{"checker_callstate", single<CallStateChecker>},
	{"printer_schema", single<SchemaPrinter>},
	{"printer_tuplecount", single<TupleCountPrinter>},
	{"printer_perfcount", single<PerfCountPrinter>},
	{"sort", single<SortLimit>},
	{"printer_bitentropy", single<BitEntropyPrinter>},
	{"consumer", single<ConsumeOp>},
	{"printer_callcount", single<CallCountPrinter>},
	{"threadidprepend", single<ThreadIdPrependOp>},
	{"partition", single<PartitionOp>},
	{"gpupartition", single<pythia_gpu_ops::GpuPartitionOp>},
	{"gpuaggregate_sum", single<pythia_gpu_ops::GpuAggregateSumOp>},
	{"gpuaggregate_count", single<pythia_gpu_ops::GpuAggregateCountOp>},
	{"gpufilter", single<pythia_gpu_ops::GpuFilterOp>},
	{"gpuproject", single<pythia_gpu_ops::GpuProjectOp>},
};

template <class K, int N>
const K* find_kind(const K (&kinds)[N], const std::string& type)
{
	for (int i = 0; i < N; ++i)
		if (type == kinds[i].type) return &kinds[i];
	return 0;
}

// The plan node named by `ref`'s `key` entry ({name = "..."}): it must exist at
// the top level of the plan and have a type.
libconfig::Setting& child_ref(libconfig::Config& cfg, libconfig::Setting& ref, const char* key)
{
	if (!ref.exists(key))
		throw MissingParameterException(std::string("Cannot find the `") + key + "' entry of a plan node.");
	libconfig::Setting& c = ref[key];
	if (!c.exists("name"))
		throw MissingParameterException(std::string("The `") + key + "' entry of a plan node has no `name'.");
	std::string name = c["name"];
	if (!cfg.getRoot().exists(name))
		throw MissingParameterException("Cannot find the description of node `" + name + "'.");
	if (!cfg.getRoot()[name].exists("type"))
		throw MissingParameterException("Cannot find the mandatory `type' of node `" + name + "'.");
	return c;
}

void build(libconfig::Config& cfg, libconfig::Setting& ref, Operator** out, Query::UserDefinedOpMapT& udops,
		int depth, Query::OperatorDepthT& depths)
{
	std::string name = ref["name"];
	std::string type = cfg.getRoot()[name]["type"];
	Operator* op = 0;
	if (const ScanKind* k = find_kind(scans, type)) {
		op = k->make();
		*out = op;
		depths[op] = depth;
	} else if (const DualKind* k = find_kind(duals, type)) {
		DualInputOp* d = k->make();
		op = d;
		*out = op;
		depths[op] = depth;
		build(cfg, child_ref(cfg, ref, "build"), &d->buildOp, udops, depth + 1, depths);
		build(cfg, child_ref(cfg, ref, "probe"), &d->probeOp, udops, depth + 1, depths);
	} else {
		SingleInputOp* s = 0;
		if (const SingleKind* k = find_kind(singles, type)) {
			s = k->make();
		} else {
			Query::UserDefinedOpMapT::iterator it = udops.find(type);
			if (it == udops.end() || it->second == 0)
				throw MissingParameterException("`" + type + "' is neither a built-in nor a user-defined type.");
			s = it->second;
			it->second = 0;       // the query owns it now
		}
		op = s;
		*out = op;
		depths[op] = depth;
		build(cfg, child_ref(cfg, ref, "input"), &s->nextOp, udops, depth + 1, depths);
	}
	op->init(cfg, cfg.lookup(name));
}

}  // namespace

void Query::create(libconfig::Config& cfg, UserDefinedOpMapT& udops)
{
	build(cfg, child_ref(cfg, cfg.getRoot(), "treeroot"), &tree, udops, 0, operatorDepth);
}

int Query::getOperatorDepth(Operator* op)
{
	OperatorDepthT::iterator it = operatorDepth.find(op);
	return it == operatorDepth.end() ? -1 : it->second;
}
