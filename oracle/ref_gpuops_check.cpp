// Test infrastructure, not product code. Links the GPU operators
// (pythia_gb300/gpuops/gpuops.cpp compiled against the reference engine's own
// headers) and this repository's plan factory (pythia_gb300/gpuops/
// query_factory.cpp, in place of the engine's query.o) with the reference
// engine's objects, and builds plans through the engine's own Query
// (query.h:40-135): Query::create, threadInit, scanStart, getNext, scanStop.
//
// Plans, each over generator_int sources (operators/generator_int.cpp: an int
// column counting 1..N, then padding to the tuple width):
//   * hashjoin (the engine's own HashJoinOp): 65,536 build tuples x 131,072
//     probe tuples on the int column -> 65,536 rows of (B$0, P$0);
//   * the same plan with type gpuhashjoin, and with type gpumpsmjoin (with
//     buildpresorted / probepresorted: the generators' keys are sorted);
//   * gpuaggregate_count with `fields = ()` over one generator, built as a
//     registered type and as a user-defined type (query.h:106).
// With a GPU every plan must give the engine's answer; without one each GPU
// plan must still be constructed and initialised by the engine, and its
// scanStart must return Error (the GPU path has no CPU fallback). Prints one
// line per plan and exits 0 when every behaviour is the expected one.
#include <cstdio>
#include <iostream>
#include <string>

#include "libconfig.h++"
#include "query.h"
#include "operators/operators.h"
#include "visitors/allvisitors.h"

#include "gpuops.h"

using namespace libconfig;

static void generator(Config& cfg, const char* name, int mb)
{
	Setting& g = cfg.getRoot().add(name, Setting::TypeGroup);
	g.add("type", Setting::TypeString) = "generator_int";
	g.add("sizeinmb", Setting::TypeInt) = mb;
	g.add("width", Setting::TypeInt) = 16;
}

// The plan's tree lives under `treeroot`, apart from the node descriptions:
// {name = "..."; input = {...}} or {name = "..."; build = {...}; probe = {...}}.
static Setting& child(Setting& ref, const char* key, const char* target)
{
	Setting& c = ref.add(key, Setting::TypeGroup);
	c.add("name", Setting::TypeString) = target;
	return c;
}

// Join of a 1 MB and a 2 MB generator on their int column, rows (B$0, P$0).
static void join_plan(Config& cfg, const std::string& type)
{
	cfg.getRoot().add("buffsize", Setting::TypeInt) = 1 << 16;
	generator(cfg, "gb", 1);
	generator(cfg, "gp", 2);
	Setting& j = cfg.getRoot().add("join", Setting::TypeGroup);
	j.add("type", Setting::TypeString) = type;
	Setting& h = j.add("hash", Setting::TypeGroup);
	h.add("fn", Setting::TypeString) = "modulo";
	h.add("buckets", Setting::TypeInt) = 1 << 16;
	j.add("tuplesperbucket", Setting::TypeInt) = 4;
	j.add("allocpolicy", Setting::TypeString) = "local";
	j.add("buildjattr", Setting::TypeInt) = 0;
	j.add("probejattr", Setting::TypeInt) = 0;
	Setting& p = j.add("projection", Setting::TypeList);
	p.add(Setting::TypeString) = "B$0";
	p.add(Setting::TypeString) = "P$0";
	Setting& tg = j.add("threadgroups", Setting::TypeList).add(Setting::TypeArray);
	tg.add(Setting::TypeInt) = 0;
	if (type == "gpumpsmjoin") {
		j.add("maxbuildtuplesinM", Setting::TypeInt) = 1;
		j.add("maxprobetuplesinM", Setting::TypeInt) = 1;
		j.add("buildpresorted", Setting::TypeString) = "yes";
		j.add("probepresorted", Setting::TypeString) = "yes";
	}
	Setting& root = child(cfg.getRoot(), "treeroot", "join");
	child(root, "build", "gb");
	child(root, "probe", "gp");
}

static void count_plan(Config& cfg, const std::string& type)
{
	cfg.getRoot().add("buffsize", Setting::TypeInt) = 1 << 16;
	generator(cfg, "gen", 1);
	Setting& agg = cfg.getRoot().add("agg", Setting::TypeGroup);
	agg.add("type", Setting::TypeString) = type;
	agg.add("fields", Setting::TypeList);
	child(child(cfg.getRoot(), "treeroot", "agg"), "input", "gen");
}

// Runs the plan; rows = output tuples, sum = sum of column 0 (int for joins,
// long for the count). Returns 1 for Error at scanStart, 0 otherwise.
static int run(Query& q, bool int_col, long long* rows, long long* sum, std::string* why)
{
	q.threadInit();
	*rows = 0; *sum = 0;
	int err = 0;
	if (q.scanStart() != Operator::Ready) {
		*why = pythia_gpu_ops::last_failure();
		err = 1;
	} else {
		Operator::GetNextResultT r;
		do {
			r = q.getNext();
			if (r.first == Operator::Error) { err = 2; break; }
			void* t;
			for (int i = 0; (t = r.second->getTupleOffset(i)); ++i) {
				++*rows;
				*sum += int_col ? *(int*) t : *(long long*) t;
			}
		} while (r.first == Operator::Ready);
		q.scanStop();
	}
	q.threadClose();
	q.destroy();
	return err;
}

int main()
{
	const bool gpu = pythia_gpu_ops::shared_context() != 0;
	const long long nb = 1024LL * 1024 / 16, want_sum = nb * (nb + 1) / 2;
	int failures = 0;
	const char* joins[] = {"hashjoin", "gpuhashjoin", "gpumpsmjoin"};
	for (int k = 0; k < 3; ++k) {
		Config cfg;
		join_plan(cfg, joins[k]);
		Query q;
		q.create(cfg);
		const bool is_gpu = joins[k][0] == 'g';
		const int depth = q.getOperatorDepth(q.tree);
		long long rows, sum;
		std::string why;
		const int err = run(q, true, &rows, &sum, &why);
		bool ok;
		if (is_gpu && !gpu) {
			ok = err == 1 && depth == 0;
			std::cout << joins[k] << ": constructed by Query::create, scanStart Error without a GPU (" << why << ")";
		} else {
			ok = err == 0 && rows == nb && sum == want_sum && depth == 0;
			std::cout << joins[k] << ": rows " << rows << " want " << nb << ", sum " << sum << " want " << want_sum;
		}
		std::cout << (ok ? "  ok" : "  FAILED") << std::endl;
		failures += !ok;
	}
	for (int k = 0; k < 2; ++k) {
		Config cfg;
		count_plan(cfg, "gpuaggregate_count");
		Query q;
		Query::UserDefinedOpMapT udops;
		if (k == 1) {
			// The registered name given as a user-defined type instead.
			cfg.getRoot()["agg"]["type"] = "my_gpu_count";
			udops["my_gpu_count"] = new pythia_gpu_ops::GpuAggregateCountOp();
		}
		q.create(cfg, udops);
		long long rows, sum;
		std::string why;
		const int err = run(q, false, &rows, &sum, &why);
		const bool ok = gpu ? (err == 0 && rows == 1 && sum == nb) : err == 1;
		std::cout << (k ? "user-defined " : "") << "gpuaggregate_count: ";
		if (gpu) std::cout << "count " << sum << " want " << nb;
		else std::cout << "scanStart Error without a GPU (" << why << ")";
		std::cout << (ok ? "  ok" : "  FAILED") << std::endl;
		failures += !ok;
	}
	return failures ? 1 : 0;
}
