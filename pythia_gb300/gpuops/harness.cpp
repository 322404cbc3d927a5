// Plan runner for the GPU operators on the mirror interface: the parity tests
// and drivers use it where the Pythia engine is not built. It plays the
// engine's parts around the operators:
//
//  * MemScanOp ("memscan"): a ZeroInputOp over a relation registered from the
//    caller's memory; thread t of T reads rows [t n / T, (t + 1) n / T) as
//    pages of `buffsize` bytes, like ParallelScanOp's per-thread files;
//  * plan construction as Query::create / constructsubtree do it
//    (query.cpp:62-233): `treeroot` names the root node, every node is a
//    top-level group with `type`, a SingleInputOp's child is its `input`, a
//    DualInputOp's its `build` and `probe`; children are initialised first;
//  * execution as the engine's threads do: every thread calls threadInit on
//    every operator, scanStart on the root, getNext until Finished, scanStop,
//    threadClose; then destroy.
//
// C entry points (pgo_*) expose registration and execution to ctypes.
#include "gpuops.h"

#include <cstdlib>
#include <cstring>
#include <map>
#include <sstream>
#include <stdexcept>

namespace {

struct Relation { const char* data; unsigned long long n; unsigned width; };
pthread_mutex_t g_rel_mu = PTHREAD_MUTEX_INITIALIZER;
std::map<std::string, Relation> g_relations;

class MemScanOp : public ZeroInputOp {
public:
	MemScanOp() : threads_(1) { rel_.data = 0; rel_.n = 0; rel_.width = 0; }
	virtual void init(libconfig::Config& root, libconfig::Setting& node)
	{
		Operator::init(root, node);
		schema = Schema::create(node["schema"]);
		std::string name = node["relation"];
		pthread_mutex_lock(&g_rel_mu);
		std::map<std::string, Relation>::iterator it = g_relations.find(name);
		const bool found = it != g_relations.end();
		if (found) rel_ = it->second;
		pthread_mutex_unlock(&g_rel_mu);
		if (!found) throw std::invalid_argument("memscan: relation `" + name + "' not registered");
		if (rel_.width != schema.getTupleSize()) throw std::invalid_argument("memscan: schema width mismatch");
		threads_ = (int) root.getRoot()["threads"];
		page_bytes_ = std::max(rel_.width, buffsize / std::max(rel_.width, 1u) * rel_.width);
		at_.assign(MAX_THREADS, 0);
		end_.assign(MAX_THREADS, 0);
		page_.assign(MAX_THREADS, (Page*) 0);
	}
	virtual ResultCode scanStart(unsigned short tid, Page* idx, Schema& idxs)
	{
		(void) idx; (void) idxs;
		if (tid >= threads_) return Error;
		at_[tid] = rel_.n * tid / threads_;
		end_[tid] = rel_.n * (tid + 1) / threads_;
		return Ready;
	}
	virtual GetNextResultT getNext(unsigned short tid)
	{
		delete page_[tid];
		const unsigned long long rows = std::min<unsigned long long>(end_[tid] - at_[tid], page_bytes_ / rel_.width);
		char* p = (char*) rel_.data + at_[tid] * rel_.width;
		page_[tid] = new Page(p, rows * rel_.width, p + rows * rel_.width, rel_.width);
		at_[tid] += rows;
		return std::make_pair(at_[tid] == end_[tid] ? Finished : Ready, page_[tid]);
	}
	virtual void threadClose(unsigned short tid) { delete page_[tid]; page_[tid] = 0; }
private:
	Relation rel_;
	unsigned threads_;
	unsigned page_bytes_;
	std::vector<unsigned long long> at_, end_;
	std::vector<Page*> page_;
};

Operator* build_tree(libconfig::Config& cfg, libconfig::Setting& ref, std::vector<Operator*>& all)
{
	std::string name = ref["name"];
	libconfig::Setting& node = cfg.getRoot()[name];
	std::string type = node["type"];
	Operator* op = 0;
	if (type == "memscan") op = new MemScanOp();
	else op = pythia_gpu_ops::create(type);
	if (!op) throw std::invalid_argument("`" + type + "' is not a GPU operator type");
	all.push_back(op);
	if (DualInputOp* d = dynamic_cast<DualInputOp*>(op)) {
		d->buildOp = build_tree(cfg, ref["build"], all);
		d->probeOp = build_tree(cfg, ref["probe"], all);
	} else if (SingleInputOp* s = dynamic_cast<SingleInputOp*>(op)) {
		s->nextOp = build_tree(cfg, ref["input"], all);
	}
	op->init(cfg, node);
	return op;
}

struct Run {
	Operator* root;
	std::vector<Operator*>* all;
	int tid;
	int rc;
	std::vector<char> out;
};

void* run_thread(void* arg)
{
	Run* r = (Run*) arg;
	const unsigned short tid = (unsigned short) r->tid;
	for (size_t i = 0; i < r->all->size(); ++i) (*r->all)[i]->threadInit(tid);
	Schema empty;
	if (r->root->scanStart(tid, 0, empty) != Operator::Ready) { r->rc = 1; }
	else {
		for (;;) {
			Operator::GetNextResultT g = r->root->getNext(tid);
			if (g.first == Operator::Error) { r->rc = 1; break; }
			if (g.second && g.second->getUsedSpace()) {
				const char* b = (const char*) g.second->getTupleOffset(0);
				r->out.insert(r->out.end(), b, b + g.second->getUsedSpace());
			}
			if (g.first == Operator::Finished) {
				// Finished repeats.
				if (r->root->getNext(tid).first != Operator::Finished) r->rc = 3;
				break;
			}
		}
		if (r->root->scanStop(tid) == Operator::Error) r->rc = 1;
	}
	for (size_t i = 0; i < r->all->size(); ++i) (*r->all)[i]->threadClose(tid);
	return 0;
}

void set_err(char* err, int errlen, const std::string& msg)
{
	if (err && errlen > 0) {
		strncpy(err, msg.c_str(), (size_t) errlen - 1);
		err[errlen - 1] = 0;
	}
}

}  // namespace

extern "C" {

// Registers (or replaces) an in-memory relation of n tuples of `width` bytes
// for memscan nodes; the memory must outlive the plans that read it.
int pgo_register(const char* name, const void* data, unsigned long long n, unsigned width)
{
	if (!name || (n && !data) || !width) return 1;
	Relation r;
	r.data = (const char*) data; r.n = n; r.width = width;
	pthread_mutex_lock(&g_rel_mu);
	g_relations[name] = r;
	pthread_mutex_unlock(&g_rel_mu);
	return 0;
}

// Runs the plan in libconfig text with `threads` threads (root key "threads"
// is set to it). Output: a malloc'd buffer of all threads' tuples in thread
// order (*out, free with pgo_free), its size, the output tuple width and the
// bytes each thread returned (thread_bytes, `threads` entries, may be NULL).
// Returns 0, 1 when an operator returned Error, 2 for a plan the operators
// refused (message in err), 3 when getNext did not repeat Finished.
int pgo_run(const char* plan, int threads, void** out, unsigned long long* nbytes, unsigned* tuple_size,
		unsigned long long* thread_bytes, char* err, int errlen)
{
	if (!plan || !out || !nbytes || !tuple_size || threads < 1 || threads > MAX_THREADS) return 2;
	*out = 0; *nbytes = 0; *tuple_size = 0;
	libconfig::Config cfg;
	std::vector<Operator*> all;
	Operator* root = 0;
	try {
		cfg.readString(plan);
		if (cfg.getRoot().exists("threads")) {
			cfg.getRoot()["threads"] = threads;
		} else {
			cfg.getRoot().add("threads", libconfig::Setting::TypeInt) = threads;
		}
		root = build_tree(cfg, cfg.getRoot()["treeroot"], all);
	} catch (const std::exception& e) {
		for (size_t i = 0; i < all.size(); ++i) delete all[i];
		set_err(err, errlen, e.what());
		return 2;
	}
	std::vector<Run> runs(threads);
	std::vector<pthread_t> th(threads);
	int rc = 0;
	try {
		for (int t = 0; t < threads; ++t) {
			runs[t].root = root; runs[t].all = &all; runs[t].tid = t; runs[t].rc = 0;
			pthread_create(&th[t], 0, run_thread, &runs[t]);
		}
		for (int t = 0; t < threads; ++t) pthread_join(th[t], 0);
	} catch (const std::exception& e) {
		set_err(err, errlen, e.what());
		rc = 2;
	}
	unsigned long long total = 0;
	for (int t = 0; t < threads; ++t) {
		if (runs[t].rc && !rc) rc = runs[t].rc;
		total += runs[t].out.size();
		if (thread_bytes) thread_bytes[t] = runs[t].out.size();
	}
	if (rc == 1) set_err(err, errlen, pythia_gpu_ops::last_failure());
	char* buf = (char*) malloc(total ? total : 1);
	unsigned long long o = 0;
	for (int t = 0; t < threads; ++t) {
		if (!runs[t].out.empty()) memcpy(buf + o, &runs[t].out[0], runs[t].out.size());
		o += runs[t].out.size();
	}
	*out = buf;
	*nbytes = total;
	*tuple_size = root->getOutSchema().getTupleSize();
	for (size_t i = 0; i < all.size(); ++i) all[i]->destroy();
	for (size_t i = 0; i < all.size(); ++i) delete all[i];
	return rc;
}

void pgo_free(void* p) { free(p); }

// Page-locks (pin = 1) or releases (pin = 0) the memory of a registered
// relation, as a loader that reads tables into pinned memory would leave
// it: GPU operators then copy its pages to the device directly. Returns 0,
// or 1 when the relation is unknown or the GPU call failed.
int pgo_pin(const char* name, int pin)
{
	pthread_mutex_lock(&g_rel_mu);
	std::map<std::string, Relation>::iterator it = g_relations.find(name ? name : "");
	const bool found = it != g_relations.end();
	Relation r = found ? it->second : Relation();
	pthread_mutex_unlock(&g_rel_mu);
	if (!found) return 1;
	pg_ctx* ctx = pythia_gpu_ops::shared_context();
	if (!ctx || !r.data || !r.n) return ctx ? 0 : 1;
	const int rc = pin ? pg_host_register(ctx, (void*) r.data, r.n * r.width) : pg_host_unregister(ctx, (void*) r.data);
	return rc ? 1 : 0;
}

// Bytes the GPU operators moved since the last reset: out[0] pages uploaded,
// out[1] outputs downloaded, out[2] device copies gathering inputs, out[3]
// inputs taken on the device in place (a count), out[4] of out[0] the bytes
// copied straight from pinned or registered pages.
void pgo_transfer_stats(unsigned long long* out)
{
	const pythia_gpu_ops::TransferStats t = pythia_gpu_ops::transfer_stats();
	out[0] = t.h2d; out[1] = t.d2h; out[2] = t.d2d; out[3] = t.in_place; out[4] = t.direct;
}

void pgo_reset_transfer_stats() { pythia_gpu_ops::reset_transfer_stats(); }

// 1 (default): adjacent GPU operators exchange data on the device; 0: every
// operator reads and writes host pages.
void pgo_set_device_exchange(int on) { pythia_gpu_ops::set_device_exchange(on != 0); }

// Phase trace of the GPU operators: pgo_trace(1) empties the ring and turns
// it on, pgo_trace(0) turns it off; pgo_trace_dump copies "ns node thread
// phase" lines into buf (NUL-terminated, truncated to len) and returns the
// bytes the whole dump needs.
void pgo_trace(int on) { pythia_gpu_ops::trace_enable(on != 0); }

unsigned long long pgo_trace_dump(char* buf, unsigned long long len) { return pythia_gpu_ops::trace_dump(buf, len); }

}  // extern "C"
