// Test infrastructure (oracle side): runs the REFERENCE Pythia operators
// (compiled unmodified from the reference source tree by oracle/Makefile.ref)
// on binary relation files and writes their output rows to a binary file.
//
// It exists to pin oracle/pythia_oracle.c (the C restatement) and to make the
// golden fixtures under tests/golden/. Nothing in the product links it.
//
// Plans are built programmatically the way the reference's own unit tests do
// (unit_tests/queryhashjoin.cpp:118-200, unit_tests/queryaggsum.cpp:110-170,
// unit_tests/querypartition.cpp:141-200, unit_tests/querympsmpkfkjoin.cpp:149-230):
// a libconfig::Config is filled node by node, the tree is wired by hand and each
// node's init(cfg, node) is called bottom-up. Input comes from MemScan, an
// in-memory ZeroInputOp written here that hands each worker thread its
// contiguous slice of the relation as zero-copy pages (as PartitionOp::getNext
// does, operators/partition.cpp:377-404).
//
// usage: ref_driver <mode> key=value ...
//   modes: hashjoin partition aggsum aggcount mpsm oldmpsm sort
//   writes the output rows to out=PATH and one JSON line to stdout.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include <map>
#include <sstream>
#include <time.h>

#include "libconfig.h++"
#include "query.h"
#include "operators/operators.h"
#include "visitors/allvisitors.h"

using namespace std;
using namespace libconfig;

static map<string, string> args;

static string arg(const char* k, const char* dflt = 0)
{
	map<string, string>::iterator it = args.find(k);
	if (it == args.end()) {
		if (!dflt) { fprintf(stderr, "missing argument %s\n", k); exit(2); }
		return dflt;
	}
	return it->second;
}
static long long argl(const char* k, const char* dflt = 0) { return atoll(arg(k, dflt).c_str()); }

static vector<string> split(const string& s)
{
	vector<string> r; string cur; stringstream ss(s);
	while (getline(ss, cur, ',')) if (!cur.empty()) r.push_back(cur);
	return r;
}

struct Relation {
	char* data; unsigned long long bytes; unsigned int tuplesize;
};

static Relation loadrel(const string& path, unsigned int tuplesize)
{
	Relation r; r.tuplesize = tuplesize;
	FILE* f = fopen(path.c_str(), "rb");
	if (!f) { fprintf(stderr, "cannot open %s\n", path.c_str()); exit(2); }
	fseek(f, 0, SEEK_END); r.bytes = ftell(f); fseek(f, 0, SEEK_SET);
	r.data = (char*) aligned_alloc(64, r.bytes + 64);
	if (r.bytes && fread(r.data, 1, r.bytes, f) != r.bytes) { fprintf(stderr, "short read\n"); exit(2); }
	fclose(f);
	return r;
}

// Zero-input operator serving a memory-resident relation: thread t gets tuples
// [t*n/T, (t+1)*n/T) in pages of at most buffsize bytes.
class MemScan : public ScanOp {
public:
	Relation rel; int threads;
	vector<unsigned long long> pos, end;
	vector<Page*> pages;

	void init(Config& root, Setting& node) {
		Operator::init(root, node);
		Setting& s = node["schema"];
		schema = Schema::create(s);
		for (int i = 0; i < MAX_THREADS; ++i) { pos.push_back(0); end.push_back(0); pages.push_back(0); }
	}
	void threadInit(unsigned short tid) { pages[tid] = new Page(0, 0, 0, rel.tuplesize); }
	ResultCode scanStart(unsigned short tid, Page*, Schema&) {
		unsigned long long n = rel.bytes / rel.tuplesize;
		pos[tid] = n * tid / threads; end[tid] = n * (tid + 1) / threads;
		if (tid >= threads) pos[tid] = end[tid] = n;
		return Ready;
	}
	GetNextResultT getNext(unsigned short tid) {
		unsigned long long per = buffsize / rel.tuplesize; if (per == 0) per = 1;
		unsigned long long take = end[tid] - pos[tid];
		ResultCode rc = Finished;
		if (take > per) { take = per; rc = Ready; }
		char* start = rel.data + pos[tid] * rel.tuplesize;
		*pages[tid] = Page(start, take * rel.tuplesize, 0, rel.tuplesize);
		pos[tid] += take;
		return make_pair(rc, pages[tid]);
	}
	ResultCode scanStop(unsigned short) { return Ready; }
	void threadClose(unsigned short tid) { delete pages[tid]; pages[tid] = 0; }
	void destroy() { }
};

static void addschema(Setting& parent, const string& schema)
{
	Setting& s = parent.add("schema", Setting::TypeList);
	vector<string> cols = split(schema);
	for (size_t i = 0; i < cols.size(); ++i) s.add(Setting::TypeString) = cols[i];
}

// Tuple width of a schema list: int 4, char(N) N + 1 (Schema::create,
// schema.cpp:221-259), everything else 8.
static unsigned int schemawidth(const string& schema)
{
	vector<string> cols = split(schema); unsigned int w = 0;
	for (size_t i = 0; i < cols.size(); ++i) {
		if (cols[i] == "int") w += 4;
		else if (cols[i].compare(0, 5, "char(") == 0) w += atoi(cols[i].c_str() + 5) + 1;
		else w += 8;
	}
	return w;
}

static double now_s()
{
	timespec ts; clock_gettime(CLOCK_MONOTONIC, &ts);
	return ts.tv_sec + ts.tv_nsec * 1e-9;
}

static void addthreadgroup(Setting& node, int threads)
{
	Setting& pg = node.add("threadgroups", Setting::TypeList);
	Setting& g = pg.add(Setting::TypeArray);
	for (int i = 0; i < threads; ++i) g.add(Setting::TypeInt) = i;
}

// Runs q to completion, returns seconds; appends all output rows to out.
static double runquery(Query& q, vector<char>& out)
{
	q.threadInit();
	double t0 = now_s();
	Operator::ResultCode sc = q.scanStart();
	if (sc == Operator::Error) { fprintf(stderr, "scanStart failed\n"); exit(3); }
	Operator::GetNextResultT r;
	do {
		r = q.getNext();
		if (r.first == Operator::Error) { fprintf(stderr, "getNext error\n"); exit(3); }
		Operator::Page* p = r.second;
		unsigned long long used = p->getUsedSpace();
		if (used) {
			char* d = (char*) p->getTupleOffset(0);
			out.insert(out.end(), d, d + used);
		}
	} while (r.first == Operator::Ready);
	if (q.scanStop() == Operator::Error) { fprintf(stderr, "scanStop failed\n"); exit(3); }
	double t1 = now_s();
	q.threadClose();
	return t1 - t0;
}

static void writeout(const vector<char>& out)
{
	string path = arg("out", "");
	if (path.empty()) return;
	FILE* f = fopen(path.c_str(), "wb");
	if (!out.empty()) fwrite(&out[0], 1, out.size(), f);
	fclose(f);
}

int main(int argc, char** argv)
{
	if (argc < 2) { fprintf(stderr, "usage: ref_driver mode k=v...\n"); return 2; }
	string mode = argv[1];
	for (int i = 2; i < argc; ++i) {
		string a = argv[i]; size_t e = a.find('=');
		if (e == string::npos) { fprintf(stderr, "bad arg %s\n", argv[i]); return 2; }
		args[a.substr(0, e)] = a.substr(e + 1);
	}
	int threads = argl("threads", "4");
	int buffsize = argl("buffsize", "1048576");
	int reps = argl("reps", "1");

	Config cfg;
	cfg.getRoot().add("path", Setting::TypeString) = "./";
	cfg.getRoot().add("buffsize", Setting::TypeInt) = buffsize;
	Setting& mergenode = cfg.getRoot().add("merge", Setting::TypeGroup);
	mergenode.add("threads", Setting::TypeInt) = threads;

	vector<char> out;
	double best = 1e30;
	unsigned long long intuples = 0;

	if (mode == "sort") {
		// TupleBuffer::sort<CtLong> over one page (util/buffer.inl:135-292), the
		// sort SortMergeJoinOp/PartitionOp use through sortAllInPage.
		string schema = arg("schema", "long,long");
		Relation r = loadrel(arg("in"), schemawidth(schema));
		intuples = r.bytes / r.tuplesize;
		for (int k = 0; k < reps; ++k) {
			vector<char> copy(r.data, r.data + r.bytes);
			Operator::Page page(copy.empty() ? 0 : &copy[0], r.bytes, 0, r.tuplesize);
			double t0 = now_s();
			page.sort<CtLong>((unsigned int) argl("keyoff", "0"));
			double t = now_s() - t0; if (t < best) best = t;
			out.assign(copy.begin(), copy.end());
		}
	}
	else if (mode == "hashjoin" || mode == "mpsm" || mode == "oldmpsm") {
		string bs = arg("bschema", "long,long"), ps = arg("pschema", "long,long");
		Relation R = loadrel(arg("build"), schemawidth(bs));
		Relation S = loadrel(arg("probe"), schemawidth(ps));
		intuples = R.bytes / R.tuplesize + S.bytes / S.tuplesize;
		for (int k = 0; k < reps; ++k) {
			Setting& root = cfg.getRoot();
			if (root.exists("scan1")) { root.remove("scan1"); root.remove("scan2"); root.remove("join"); }
			if (root.exists("aggpre")) { root.remove("aggpre"); root.remove("aggpost"); }
			Setting& s1 = root.add("scan1", Setting::TypeGroup); addschema(s1, bs);
			Setting& s2 = root.add("scan2", Setting::TypeGroup); addschema(s2, ps);
			Setting& jn = root.add("join", Setting::TypeGroup);
			addthreadgroup(jn, threads);
			jn.add("buildjattr", Setting::TypeInt) = (int) argl("buildjattr", "0");
			jn.add("probejattr", Setting::TypeInt) = (int) argl("probejattr", "0");
			Setting& proj = jn.add("projection", Setting::TypeList);
			vector<string> pj = split(arg("proj", "P$1,B$1"));
			for (size_t i = 0; i < pj.size(); ++i) proj.add(Setting::TypeString) = pj[i];

			MemScan b, p; b.rel = R; b.threads = threads; p.rel = S; p.threads = threads;
			MergeOp merge;
			HashJoinOp hj; MPSMJoinOp mj; OldMPSMJoinOp omj;
			DualInputOp* join;
			if (mode == "hashjoin") {
				Setting& h = jn.add("hash", Setting::TypeGroup);
				h.add("fn", Setting::TypeString) = arg("fn", "modulo");
				h.add("buckets", Setting::TypeInt) = (int) argl("buckets", "1048576");
				if (args.count("min")) {
					Setting& rg = h.add("range", Setting::TypeArray);
					rg.add(Setting::TypeInt) = (int) argl("min");
					rg.add(Setting::TypeInt) = (int) argl("max");
				}
				jn.add("tuplesperbucket", Setting::TypeInt) = (int) argl("tuplesperbucket", "4");
				jn.add("allocpolicy", Setting::TypeString) = "local";
				join = &hj;
			} else {
				jn.add("maxbuildtuples", Setting::TypeInt) = (int) argl("maxbuildtuples", "0");
				jn.add("maxprobetuples", Setting::TypeInt) = (int) argl("maxprobetuples", "0");
				jn.add("mostfreqbuildkeyoccurances", Setting::TypeInt) = (int) argl("mostfreq", "1");
				join = (mode == "mpsm") ? (DualInputOp*) &mj : (DualInputOp*) &omj;
			}
			join->buildOp = &b; join->probeOp = &p;
			b.init(cfg, s1); p.init(cfg, s2);
			join->init(cfg, jn);

			// Optional global (no GROUP BY) count or sum over the join output,
			// two-stage as the reference tests do: per-thread aggregate, merge,
			// then one aggregate summing the partials.
			string agg = arg("agg", "none");
			Query q;
			AggregateCount cnt; AggregateSum pre, post;
			if (agg == "none") {
				merge.nextOp = join; merge.init(cfg, mergenode); q.tree = &merge;
			} else {
				Setting& an = root.add("aggpre", Setting::TypeGroup);
				an.add("fields", Setting::TypeArray);
				Setting& pn = root.add("aggpost", Setting::TypeGroup);
				pn.add("fields", Setting::TypeArray);
				pn.add("sumfield", Setting::TypeInt) = 0;
				GenericAggregate* lower;
				if (agg == "count") { lower = &cnt; }
				else { an.add("sumfield", Setting::TypeInt) = (int) argl("sumfield", "1"); lower = &pre; }
				lower->nextOp = join; lower->init(cfg, an);
				merge.nextOp = lower; merge.init(cfg, mergenode);
				post.nextOp = &merge; post.init(cfg, pn);
				q.tree = &post;
			}
			out.clear();
			double t = runquery(q, out); if (t < best) best = t;
			q.destroynofree();
		}
	}
	else if (mode == "partition") {
		string schema = arg("schema", "long,long");
		Relation R = loadrel(arg("in"), schemawidth(schema));
		intuples = R.bytes / R.tuplesize;
		for (int k = 0; k < reps; ++k) {
			Setting& root = cfg.getRoot();
			if (root.exists("scan")) { root.remove("scan"); root.remove("part"); root.remove("tidp"); }
			Setting& s = root.add("scan", Setting::TypeGroup); addschema(s, schema);
			Setting& pn = root.add("part", Setting::TypeGroup);
			pn.add("attr", Setting::TypeInt) = (int) argl("attr", "0");
			pn.add("maxtuples", Setting::TypeInt) = (int) (intuples + 1024);
			Setting& rg = pn.add("range", Setting::TypeArray);
			rg.add(Setting::TypeInt) = (int) argl("min");
			rg.add(Setting::TypeInt) = (int) argl("max");
			pn.add("buckets", Setting::TypeInt) = threads;
			pn.add("sort", Setting::TypeString) = arg("sort", "no");
			Setting& tn = root.add("tidp", Setting::TypeGroup);
			MemScan sc; sc.rel = R; sc.threads = threads;
			PartitionOp part; ThreadIdPrependOp tidp; MergeOp merge;
			part.nextOp = &sc; tidp.nextOp = &part; merge.nextOp = &tidp;
			sc.init(cfg, s); part.init(cfg, pn); tidp.init(cfg, tn); merge.init(cfg, mergenode);
			Query q; q.tree = &merge;
			out.clear();
			double t = runquery(q, out); if (t < best) best = t;
			q.destroynofree();
		}
	}
	else if (mode == "aggsum" || mode == "aggcount") {
		string schema = arg("schema", "long,dec");
		Relation R = loadrel(arg("in"), schemawidth(schema));
		intuples = R.bytes / R.tuplesize;
		string aggmode = arg("aggmode", "twostage");
		for (int k = 0; k < reps; ++k) {
			Setting& root = cfg.getRoot();
			if (root.exists("scan")) { root.remove("scan"); root.remove("aggpre"); if (root.exists("aggpost")) root.remove("aggpost"); }
			Setting& s = root.add("scan", Setting::TypeGroup); addschema(s, schema);
			int field = (int) argl("field", "0");
			int buckets = (int) argl("buckets", "1048576");
			string fn = arg("fn", "modulo");
			Setting& an = root.add("aggpre", Setting::TypeGroup);
			an.add("field", Setting::TypeInt) = field;
			if (mode == "aggsum") an.add("sumfield", Setting::TypeInt) = (int) argl("sumfield", "1");
			Setting& h = an.add("hash", Setting::TypeGroup);
			h.add("fn", Setting::TypeString) = fn;
			h.add("buckets", Setting::TypeInt) = buckets;
			h.add("field", Setting::TypeInt) = field;
			MemScan sc; sc.rel = R; sc.threads = threads;
			AggregateSum s1, s2; AggregateCount c1; MergeOp merge;
			GenericAggregate* lower = (mode == "aggsum") ? (GenericAggregate*) &s1 : (GenericAggregate*) &c1;
			Query q;
			if (aggmode == "global") {
				an.add("global", Setting::TypeBoolean) = true;
				an.add("threads", Setting::TypeInt) = threads;
				lower->nextOp = &sc; merge.nextOp = lower;
				sc.init(cfg, s); lower->init(cfg, an); merge.init(cfg, mergenode);
				q.tree = &merge;
			} else {
				// Stage two sums the per-thread partials: (key, partial) rows,
				// so it is always an aggregate_sum over column 1.
				Setting& pn = root.add("aggpost", Setting::TypeGroup);
				pn.add("field", Setting::TypeInt) = 0;
				pn.add("sumfield", Setting::TypeInt) = 1;
				Setting& h2 = pn.add("hash", Setting::TypeGroup);
				h2.add("fn", Setting::TypeString) = fn;
				h2.add("buckets", Setting::TypeInt) = buckets;
				h2.add("field", Setting::TypeInt) = 0;
				lower->nextOp = &sc; merge.nextOp = lower; s2.nextOp = &merge;
				sc.init(cfg, s); lower->init(cfg, an); merge.init(cfg, mergenode); s2.init(cfg, pn);
				q.tree = &s2;
			}
			out.clear();
			double t = runquery(q, out); if (t < best) best = t;
			q.destroynofree();
		}
	}
	else if (mode == "hash") {
		// TupleHasher::create + hash over every tuple (hash.cpp:99-234),
		// output one unsigned int per tuple, then buckets() as a last word.
		string schema = arg("schema", "long,long");
		Relation R = loadrel(arg("in"), schemawidth(schema));
		intuples = R.bytes / R.tuplesize;
		Setting& s = cfg.getRoot().add("scan", Setting::TypeGroup); addschema(s, schema);
		Schema sch = Schema::create(s["schema"]);
		Setting& h = cfg.getRoot().add("hash", Setting::TypeGroup);
		h.add("fn", Setting::TypeString) = arg("fn");
		h.add("buckets", Setting::TypeInt) = (int) argl("buckets", "16");
		if (args.count("fieldmin")) {
			Setting& fr = h.add("fieldrange", Setting::TypeArray);
			fr.add(Setting::TypeInt) = (int) argl("fieldmin");
			fr.add(Setting::TypeInt) = (int) argl("fieldmax");
		} else h.add("field", Setting::TypeInt) = (int) argl("field", "0");
		if (args.count("min")) {
			Setting& rg = h.add("range", Setting::TypeArray);
			rg.add(Setting::TypeInt) = (int) argl("min");
			rg.add(Setting::TypeInt) = (int) argl("max");
		}
		if (args.count("skipbits")) h.add("skipbits", Setting::TypeInt) = (int) argl("skipbits");
		if (args.count("offset")) h.add("offset", Setting::TypeInt) = (int) argl("offset");
		TupleHasher th = TupleHasher::create(sch, h);
		out.resize((intuples + 1) * 4);
		unsigned int* o = (unsigned int*) &out[0];
		for (unsigned long long i = 0; i < intuples; ++i) o[i] = th.hash(R.data + i * R.tuplesize);
		o[intuples] = th.buckets();
		th.destroy();
	}
	else if (mode == "filter" || mode == "project") {
		// Filter (filter.cpp:37-85), or a chain of them (field2/op2/value2,
		// ...), or Project (project.cpp:37-104) over one scanning thread, so
		// the output keeps the input order. Schema columns are separated by
		// ';' here (a date format may hold commas).
		string schema = arg("schema", "long;long");
		for (size_t k = 0; k < schema.size(); ++k) if (schema[k] == ';') schema[k] = ',';
		Relation R = loadrel(arg("in"), schemawidth(schema));
		intuples = R.bytes / R.tuplesize;
		Setting& root = cfg.getRoot();
		Setting& s = root.add("scan", Setting::TypeGroup); addschema(s, schema);
		MemScan sc; sc.rel = R; sc.threads = 1;
		sc.init(cfg, s);
		Filter f[4]; Project pj;
		Operator* top = &sc;
		if (mode == "filter") {
			for (int k = 0; k < 4; ++k) {
				string sfx = k ? string(1, (char) ('1' + k)) : string();
				if (!args.count("field" + sfx)) break;
				Setting& fn = root.add("filter" + sfx, Setting::TypeGroup);
				fn.add("field", Setting::TypeInt) = (int) argl(("field" + sfx).c_str());
				fn.add("op", Setting::TypeString) = arg(("op" + sfx).c_str());
				fn.add("value", Setting::TypeString) = arg(("value" + sfx).c_str());
				f[k].nextOp = top;
				f[k].init(cfg, fn);
				top = &f[k];
			}
		} else {
			Setting& pn = root.add("project", Setting::TypeGroup);
			Setting& pl = pn.add("projection", Setting::TypeArray);
			vector<string> cols = split(arg("projection"));
			for (size_t k = 0; k < cols.size(); ++k) pl.add(Setting::TypeString) = "$" + cols[k];
			pj.nextOp = top;
			pj.init(cfg, pn);
			top = &pj;
		}
		Query q; q.tree = top;
		out.clear();
		best = runquery(q, out);
		q.destroynofree();
	}
	else { fprintf(stderr, "unknown mode %s\n", mode.c_str()); return 2; }

	writeout(out);
	printf("{\"mode\": \"%s\", \"threads\": %d, \"in_tuples\": %llu, \"out_bytes\": %llu, \"best_s\": %.6f}\n",
			mode.c_str(), threads, intuples, (unsigned long long) out.size(), best);
	return 0;
}
