// Test infrastructure, not product code. Links the GPU operators
// (pythia_gb300/gpuops/gpuops.cpp compiled against the reference engine's own
// headers) with the reference engine's objects and drives one through the
// engine's Query (query.cpp:62-233, query.h:40-115): a generator_int source
// (operators/generator_int.cpp: int column 1..N plus padding) under a
// gpuaggregate_count with `fields = ()` (one global group), registered as a
// user-defined single-input type (query.h:106). With a GPU the count must be
// N; without one the operator must return Error from scanStart (the GPU path
// has no CPU fallback). Prints one line and exits 0 when the behaviour is
// the expected one.
#include <cstdio>
#include <iostream>

#include "libconfig.h++"
#include "query.h"
#include "operators/operators.h"
#include "visitors/allvisitors.h"

#include "gpuops.h"

int main()
{
	using namespace libconfig;
	Config cfg;
	cfg.getRoot().add("buffsize", Setting::TypeInt) = 1 << 16;
	Setting& gen = cfg.getRoot().add("gen", Setting::TypeGroup);
	gen.add("type", Setting::TypeString) = "generator_int";
	gen.add("sizeinmb", Setting::TypeInt) = 1;
	gen.add("width", Setting::TypeInt) = 16;
	Setting& agg = cfg.getRoot().add("agg", Setting::TypeGroup);
	agg.add("type", Setting::TypeString) = "gpuaggregate_count";
	agg.add("fields", Setting::TypeList);
	Setting& tr = cfg.getRoot().add("treeroot", Setting::TypeGroup);
	tr.add("name", Setting::TypeString) = "agg";
	tr.add("input", Setting::TypeGroup).add("name", Setting::TypeString) = "gen";

	Query::UserDefinedOpMapT udops;
	udops["gpuaggregate_count"] = new pythia_gpu_ops::GpuAggregateCountOp();
	Query q;
	q.create(cfg, udops);
	const long long want = 1024LL * 1024 / 16;
	const bool gpu = pythia_gpu_ops::shared_context() != 0;
	q.threadInit();
	int status = 1;
	if (q.scanStart() != Operator::Ready) {
		std::cout << "scanStart: Error (" << pythia_gpu_ops::last_failure() << ")" << std::endl;
		status = gpu ? 1 : 0;
	} else {
		long long count = 0;
		Operator::GetNextResultT r;
		do {
			r = q.getNext();
			if (r.first == Operator::Error) break;
			void* t;
			for (int i = 0; (t = r.second->getTupleOffset(i)); ++i) count += *(long long*) t;
		} while (r.first == Operator::Ready);
		q.scanStop();
		std::cout << "count " << count << " want " << want << std::endl;
		status = (r.first == Operator::Finished && count == want) ? 0 : 1;
	}
	q.threadClose();
	q.destroy();
	return status;
}
