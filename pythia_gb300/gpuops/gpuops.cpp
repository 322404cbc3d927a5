// GPU operators for Pythia plans (see gpuops.h). C++98, like the engine.
#include "gpuops.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <stdexcept>
#include <time.h>

namespace pythia_gpu_ops {

// ---------------------------------------------------------------------------
// Context, failures, barrier, thread groups.
// ---------------------------------------------------------------------------
namespace {
pthread_once_t g_once = PTHREAD_ONCE_INIT;
pg_ctx* g_ctx = 0;
pthread_mutex_t g_fail_mu = PTHREAD_MUTEX_INITIALIZER;
std::string g_fail;
TransferStats g_stats = {0, 0, 0, 0, 0};
volatile int g_exchange = 1;

void count(unsigned long long* c, unsigned long long v)
{
	__sync_fetch_and_add(c, v);
}

void make_context()
{
	pg_ctx* c = 0;
	if (pg_init(0, 0, &c) == PG_OK) g_ctx = c;
	else {
		pthread_mutex_lock(&g_fail_mu);
		g_fail = std::string("pg_init: ") + pg_last_error(0);
		pthread_mutex_unlock(&g_fail_mu);
	}
}

void note_failure(const char* who, int rc)
{
	pthread_mutex_lock(&g_fail_mu);
	std::ostringstream os;
	os << who << ": status " << rc << ": " << (g_ctx ? pg_last_error(g_ctx) : "no GPU context");
	g_fail = os.str();
	pthread_mutex_unlock(&g_fail_mu);
}

// Byte offset of column `attr` in tuples of `s`.
unsigned col_offset(Schema& s, unsigned attr)
{
	return (unsigned) ((char*) s.calcOffset((void*) 0x1000, attr) - (char*) 0x1000);
}

// Key width of an integer-like column (int 4, long/date 8), or 0.
unsigned key_bytes(Schema& s, unsigned attr)
{
	const ColumnType t = s.getColumnType(attr);
	if (t == CT_INTEGER) return 4;
	if (t == CT_LONG || t == CT_DATE) return 8;
	return 0;
}

int hash_fn_code(const std::string& name)
{
	if (name == "bytes") return PG_FN_BYTES;
	if (name == "modulo") return PG_FN_MODULO;
	if (name == "range") return PG_FN_RANGE;
	if (name == "exactrange") return PG_FN_EXACTRANGE;
	if (name == "parammodulo") return PG_FN_PARAMMODULO;
	if (name == "knuth") return PG_FN_KNUTH;
	if (name == "tpchorderkey") return PG_FN_TPCHORDERKEY;
	if (name == "willis") return PG_FN_WILLIS;
	if (name == "alwayszero") return PG_FN_ALWAYSZERO;
	if (name == "tpchq1magic") return PG_FN_TPCHQ1MAGIC;
	throw std::invalid_argument("unknown hash function `" + name + "'");
}
}  // namespace

pg_ctx* shared_context()
{
	pthread_once(&g_once, make_context);
	return g_ctx;
}

std::string last_failure()
{
	pthread_mutex_lock(&g_fail_mu);
	std::string s = g_fail;
	pthread_mutex_unlock(&g_fail_mu);
	return s;
}

TransferStats transfer_stats()
{
	TransferStats t;
	t.h2d = __sync_fetch_and_add(&g_stats.h2d, 0);
	t.d2h = __sync_fetch_and_add(&g_stats.d2h, 0);
	t.d2d = __sync_fetch_and_add(&g_stats.d2d, 0);
	t.in_place = __sync_fetch_and_add(&g_stats.in_place, 0);
	t.direct = __sync_fetch_and_add(&g_stats.direct, 0);
	return t;
}

void reset_transfer_stats()
{
	__sync_lock_test_and_set(&g_stats.h2d, 0);
	__sync_lock_test_and_set(&g_stats.d2h, 0);
	__sync_lock_test_and_set(&g_stats.d2d, 0);
	__sync_lock_test_and_set(&g_stats.in_place, 0);
	__sync_lock_test_and_set(&g_stats.direct, 0);
}

void set_device_exchange(bool on)
{
	g_exchange = on ? 1 : 0;
}

namespace {
struct TraceEntry { unsigned long long ns; int tid; char node[28]; char phase[24]; };
const unsigned TRACE_CAP = 1u << 16;
volatile int g_trace_on = 0;
unsigned g_trace_n = 0;
std::vector<TraceEntry> g_trace;

unsigned long long now_ns()
{
	timespec t;
	clock_gettime(CLOCK_MONOTONIC, &t);
	return (unsigned long long) t.tv_sec * 1000000000ull + (unsigned long long) t.tv_nsec;
}
}  // namespace

void trace_enable(bool on)
{
	g_trace_on = 0;
	__sync_synchronize();
	if (on) {
		if (g_trace.size() != TRACE_CAP) g_trace.resize(TRACE_CAP);
		g_trace_n = 0;
		__sync_synchronize();
		g_trace_on = 1;
	}
}

void trace(const std::string& node, int tid, const char* phase)
{
	if (!g_trace_on) return;
	const unsigned i = __sync_fetch_and_add(&g_trace_n, 1u);
	if (i >= TRACE_CAP) return;
	TraceEntry& e = g_trace[i];
	e.ns = now_ns();
	e.tid = tid;
	strncpy(e.node, node.c_str(), sizeof(e.node) - 1);
	e.node[sizeof(e.node) - 1] = 0;
	strncpy(e.phase, phase, sizeof(e.phase) - 1);
	e.phase[sizeof(e.phase) - 1] = 0;
}

unsigned long long trace_dump(char* buf, unsigned long long len)
{
	const unsigned n = std::min(g_trace_n, TRACE_CAP);
	std::string out;
	char line[128];
	for (unsigned i = 0; i < n; ++i) {
		const TraceEntry& e = g_trace[i];
		snprintf(line, sizeof(line), "%llu %s %d %s\n", e.ns, e.node[0] ? e.node : "-", e.tid, e.phase);
		out += line;
	}
	if (buf && len) {
		const unsigned long long k = std::min<unsigned long long>(len - 1, out.size());
		memcpy(buf, out.data(), (size_t) k);
		buf[k] = 0;
	}
	return out.size() + 1;
}

void GroupBarrier::arrive()
{
	pthread_mutex_lock(&mu_);
	const unsigned phase = phase_;
	if (++waiting_ == size_) {
		waiting_ = 0;
		++phase_;
		pthread_cond_broadcast(&cv_);
	} else {
		while (phase == phase_) pthread_cond_wait(&cv_, &mu_);
	}
	pthread_mutex_unlock(&mu_);
}

void ThreadGroups::parse(libconfig::Setting& node, int default_threads)
{
	group_of.assign(MAX_THREADS, -1);
	pos_in.assign(MAX_THREADS, -1);
	members.clear();
	if (node.exists("threadgroups")) {
		libconfig::Setting& tg = node["threadgroups"];
		for (int g = 0; g < tg.getLength(); ++g) {
			members.push_back(std::vector<int>());
			for (int j = 0; j < tg[g].getLength(); ++j) {
				const int tid = tg[g][j];
				if (tid < 0 || tid >= MAX_THREADS || group_of[tid] != -1)
					throw std::invalid_argument("threadgroups: bad or repeated thread id");
				group_of[tid] = g;
				pos_in[tid] = j;
				members.back().push_back(tid);
			}
		}
	} else {
		int t = default_threads;
		node.lookupValue("threads", t);
		if (t < 1 || t > MAX_THREADS) throw std::invalid_argument("threads out of range");
		members.push_back(std::vector<int>());
		for (int tid = 0; tid < t; ++tid) { group_of[tid] = 0; pos_in[tid] = tid; members[0].push_back(tid); }
	}
}

void GroupedOutput::setup(const ThreadGroups& g, unsigned tuple_size, unsigned buffsize)
{
	clear();
	tuple_size_ = tuple_size ? tuple_size : 1;
	page_bytes_ = std::max(tuple_size_, buffsize / tuple_size_ * tuple_size_);
	out_.assign(g.members.size(), std::vector<char>());
	rows_.assign(g.members.size(), 0);
	dev_.assign(g.members.size(), (const char*) 0);
	Cursor c = { 0, 0, 0, true, 0, 0 };
	cur_.assign(MAX_THREADS, c);
}

void GroupedOutput::own_device(void* p)
{
	pthread_mutex_lock(&mu_);
	owned_.push_back(p);
	pthread_mutex_unlock(&mu_);
}

void GroupedOutput::set_device(int group, const char* data, unsigned long long rows)
{
	dev_[group] = data;
	rows_[group] = rows;
}

void GroupedOutput::assign(int tid, int group, int pos, int k)
{
	const unsigned long long rows = rows_[group];
	const unsigned long long lo = rows * pos / k, hi = rows * (pos + 1) / k;
	Cursor& c = cur_[tid];
	c.at = out_[group].empty() ? 0 : &out_[group][0] + lo * tuple_size_;
	c.left = (hi - lo) * tuple_size_;
	c.done = false;
	c.dev = dev_[group] && hi > lo ? dev_[group] + lo * tuple_size_ : 0;
	c.dev_rows = dev_[group] ? hi - lo : 0;
}

DeviceSpan GroupedOutput::share(int tid) const
{
	DeviceSpan d;
	d.data = cur_[tid].dev;
	d.rows = cur_[tid].dev_rows;
	return d;
}

Operator::GetNextResultT GroupedOutput::next(int tid)
{
	Cursor& c = cur_[tid];
	delete c.page;
	const unsigned long long bytes = std::min<unsigned long long>(c.left, page_bytes_);
	c.page = new Operator::Page(c.at, bytes, c.at ? c.at + bytes : 0, tuple_size_);
	if (c.at) c.at += bytes;
	c.left -= bytes;
	if (c.left == 0) c.done = true;
	return std::make_pair(c.done ? Operator::Finished : Operator::Ready, c.page);
}

void GroupedOutput::clear()
{
	for (size_t i = 0; i < cur_.size(); ++i) { delete cur_[i].page; cur_[i].page = 0; }
	out_.clear();
	rows_.clear();
	dev_.clear();
	pg_ctx* ctx = owned_.empty() ? 0 : shared_context();
	for (size_t i = 0; i < owned_.size(); ++i) pg_buffer_free_async(ctx, 0, owned_[i]);
	owned_.clear();
}

bool drain(Operator* child, unsigned short tid, std::vector<char>& sink)
{
	for (;;) {
		Operator::GetNextResultT r = child->getNext(tid);
		if (r.first == Operator::Error) return false;
		Operator::Page* p = r.second;
		if (p) {
			const unsigned long long used = p->getUsedSpace();
			if (used) {
				const char* base = (const char*) p->getTupleOffset(0);
				sink.insert(sink.end(), base, base + used);
			}
		}
		if (r.first == Operator::Finished) return true;
	}
}

// Pinned staging buffers shared by every operator of the process: made on
// first use, kept for later plans (pinned allocation costs milliseconds).
namespace {
const unsigned long long STAGE_BYTES = 4ull << 20;
const unsigned long long FIRST_CHUNK = 16ull << 20, LAST_CHUNK = 512ull << 20;
pthread_mutex_t g_stage_mu = PTHREAD_MUTEX_INITIALIZER;
std::vector<char*> g_stage_free;

char* stage_take(pg_ctx* ctx)
{
	pthread_mutex_lock(&g_stage_mu);
	char* p = 0;
	if (!g_stage_free.empty()) { p = g_stage_free.back(); g_stage_free.pop_back(); }
	pthread_mutex_unlock(&g_stage_mu);
	if (!p) {
		void* q = 0;
		if (pg_host_alloc(ctx, STAGE_BYTES, &q) == PG_OK) p = (char*) q;
	}
	return p;
}

void stage_give(char* p)
{
	if (!p) return;
	pthread_mutex_lock(&g_stage_mu);
	g_stage_free.push_back(p);
	pthread_mutex_unlock(&g_stage_mu);
}
}  // namespace

namespace {
pthread_mutex_t g_stream_mu = PTHREAD_MUTEX_INITIALIZER;
pg_stream g_thread_streams[MAX_THREADS];

// The stream of plan thread `tid`, made on first use and kept for the
// process. Device memory an operator frees on it in one plan run is allocated
// again on it in the next, in stream order, so the pool reuses its blocks
// instead of mapping new memory (a stream destroyed after each launch left
// 1 GB buffers that later runs did not reuse). A plan thread runs one
// operator phase at a time; plans run at the same time share the streams
// of equal thread ids, which orders their work but keeps it correct.
pg_stream thread_stream(pg_ctx* ctx, int tid)
{
	if (tid < 0 || tid >= MAX_THREADS) return 0;     // the legacy stream: ordered, still correct
	pthread_mutex_lock(&g_stream_mu);
	if (!g_thread_streams[tid]) {
		pg_stream s = 0;
		if (pg_stream_create(ctx, &s) == PG_OK) g_thread_streams[tid] = s;
	}
	const pg_stream s = g_thread_streams[tid];
	pthread_mutex_unlock(&g_stream_mu);
	return s;
}
}  // namespace

void InputSide::setup(Operator* child, const std::string& node)
{
	clear();
	node_ = node;
	dev_ = g_exchange ? dynamic_cast<DeviceProducer*>(child) : 0;
	if (dev_) dev_->keep_on_device();
	host_.assign(MAX_THREADS, std::vector<char>());
	staged_.assign(MAX_THREADS, Staged());
	DeviceSpan none = { 0, 0 };
	spans_.assign(MAX_THREADS, none);
}

bool InputSide::fetch(Operator* child, unsigned short tid)
{
	if (dev_) {
		spans_[tid] = dev_->device_share(tid);
		trace(node_, tid, "span");
		return true;
	}
	if (!shared_context()) return drain(child, tid, host_[tid]);
	trace(node_, tid, "stage start");
	const bool ok = stage(child, tid);
	trace(node_, tid, "staged");
	return ok;
}

// Sends `n` bytes at `buf` (a staging buffer, or with `sm` a page the SMs
// read in place) to the thread's device chunks, opening a new chunk when the
// current one is full.
bool InputSide::flush(pg_ctx* ctx, pg_stream st, Staged& u, const char* buf, unsigned long long n,
		unsigned long long& room, unsigned long long& next_chunk, bool sm)
{
	if (!n) return true;
	if (n > room) {
		const unsigned long long size = std::max(n, next_chunk);
		void* c = 0;
		if (pg_buffer_alloc_async(ctx, st, size, &c) != PG_OK) return false;
		u.chunks.push_back((char*) c);
		u.used.push_back(0);
		room = size;
		next_chunk = std::min(next_chunk * 2, LAST_CHUNK);
	}
	if ((sm ? pg_h2d_sm(ctx, st, u.chunks.back() + u.used.back(), buf, n)
			: pg_h2d(ctx, st, u.chunks.back() + u.used.back(), buf, n)) != PG_OK) return false;
	u.used.back() += n;
	room -= n;
	count(&g_stats.h2d, n);
	return true;
}

// Reads the child's pages into two pinned buffers in turn; a full buffer is
// sent to the thread's device chunks on its own stream while the next one
// fills. Pages the GPU can read in place (pinned or registered memory, or any
// host memory on a device with pageable-memory access) skip the buffers: a
// copy kernel reads them over the host link (181 GB/s for 1 MB pages from 16
// threads, against 117 GB/s by copy engine and 55 GB/s through the staging
// copy). Chunks grow from 16 MB, doubling up to 512 MB.
bool InputSide::stage(Operator* child, unsigned short tid)
{
	pg_ctx* ctx = shared_context();
	Staged& u = staged_[tid];
	const pg_stream st = thread_stream(ctx, tid);
	char* pin[2] = { stage_take(ctx), stage_take(ctx) };
	bool ok = pin[0] && pin[1];
	int cur = 0;
	unsigned long long fill = 0, room = 0, next_chunk = FIRST_CHUNK;
	bool in_flight[2] = { false, false };
	while (ok) {
		Operator::GetNextResultT r = child->getNext(tid);
		if (r.first == Operator::Error) { ok = false; break; }
		Operator::Page* p = r.second;
		const unsigned long long used = p ? p->getUsedSpace() : 0;
		const char* src = used ? (const char*) p->getTupleOffset(0) : 0;
		if (used && pg_host_readable(ctx, src)) {
			// A page the GPU reads in place goes to the device directly, after
			// the bytes staged before it; the copy ends before the next
			// getNext, which may reuse the page.
			ok = flush(ctx, st, u, pin[cur], fill, room, next_chunk, false) &&
				flush(ctx, st, u, src, used, room, next_chunk, true) && pg_sync(ctx, st) == PG_OK;
			fill = 0;
			in_flight[0] = in_flight[1] = false;
			count(&g_stats.direct, used);
			if (r.first == Operator::Finished) break;
			continue;
		}
		unsigned long long left = used;
		while (ok && left) {
			const unsigned long long n = std::min(left, STAGE_BYTES - fill);
			memcpy(pin[cur] + fill, src, (size_t) n);
			fill += n; src += n; left -= n;
			if (fill == STAGE_BYTES) {
				ok = flush(ctx, st, u, pin[cur], fill, room, next_chunk, false);
				in_flight[cur] = true;
				cur ^= 1;
				fill = 0;
				// The other buffer's copy must be done before it refills.
				if (ok && in_flight[cur]) { ok = pg_sync(ctx, st) == PG_OK; in_flight[0] = in_flight[1] = false; }
			}
		}
		if (r.first == Operator::Finished) break;
	}
	if (ok) ok = flush(ctx, st, u, pin[cur], fill, room, next_chunk, false);
	if (pg_sync(ctx, st) != PG_OK) ok = false;
	stage_give(pin[0]);
	stage_give(pin[1]);
	return ok;
}

int InputSide::gather(pg_ctx* ctx, pg_stream st, const std::vector<int>& members, unsigned width,
		const char** data, unsigned long long* rows, void** tmp)
{
	*data = 0; *rows = 0; *tmp = 0;
	// Pieces of the input in order: device spans of a GPU child, staged
	// chunks, or (without staging) drained host bytes.
	std::vector<const char*> at;
	std::vector<unsigned long long> bytes;
	bool host = false;
	for (size_t i = 0; i < members.size(); ++i) {
		const int t = members[i];
		if (dev_) {
			at.push_back(spans_[t].data); bytes.push_back(spans_[t].rows * width);
		} else if (!host_[t].empty()) {
			host = true;
			at.push_back(&host_[t][0]); bytes.push_back(host_[t].size());
		} else {
			for (size_t c = 0; c < staged_[t].chunks.size(); ++c) {
				at.push_back(staged_[t].chunks[c]); bytes.push_back(staged_[t].used[c]);
			}
		}
	}
	unsigned long long total = 0;
	bool run = !host;
	const char* first = 0;
	const char* end = 0;
	for (size_t i = 0; i < at.size(); ++i) {
		if (!bytes[i]) continue;
		if (!first) first = at[i];
		else if (at[i] != end) run = false;
		end = at[i] + bytes[i];
		total += bytes[i];
	}
	*rows = width ? total / width : 0;
	if (!total) return PG_OK;
	// In place when the pieces are one run that starts 16-byte aligned (the
	// alignment every operator's loads assume); copied otherwise.
	if (run && ((unsigned long long) (size_t) first & 15) == 0) {
		*data = first;
		if (dev_) count(&g_stats.in_place, 1);
		return PG_OK;
	}
	int rc = pg_buffer_alloc_async(ctx, st, total, tmp);
	char* o = (char*) *tmp;
	for (size_t i = 0; i < at.size() && !rc; ++i) {
		if (!bytes[i]) continue;
		if (host) {
			rc = pg_h2d(ctx, st, o, at[i], bytes[i]);
			count(&g_stats.h2d, bytes[i]);
		} else {
			rc = pg_d2d(ctx, st, o, at[i], bytes[i]);
			if (dev_) count(&g_stats.d2d, bytes[i]);
		}
		o += bytes[i];
	}
	*data = (const char*) *tmp;
	return rc;
}

bool InputSide::pieces(const std::vector<int>& members, unsigned width,
		std::vector<std::pair<const char*, unsigned long long> >& out) const
{
	out.clear();
	if (!width) return false;
	std::vector<std::pair<const char*, unsigned long long> > all;
	for (size_t i = 0; i < members.size(); ++i) {
		const int t = members[i];
		if (dev_) {
			if (spans_[t].rows) all.push_back(std::make_pair(spans_[t].data, spans_[t].rows));
		} else if (!host_[t].empty()) {
			return false;
		} else {
			for (size_t c = 0; c < staged_[t].chunks.size(); ++c)
				if (staged_[t].used[c])
					all.push_back(std::make_pair((const char*) staged_[t].chunks[c], staged_[t].used[c] / width));
		}
	}
	// Arrays that follow each other in memory are one piece.
	for (size_t i = 0; i < all.size(); ++i) {
		if (!out.empty() && out.back().first + out.back().second * width == all[i].first) out.back().second += all[i].second;
		else out.push_back(all[i]);
	}
	return true;
}

void InputSide::release(int tid, pg_stream st)
{
	std::vector<char>().swap(host_[tid]);
	Staged& u = staged_[tid];
	if (!u.chunks.empty()) {
		pg_ctx* ctx = shared_context();
		for (size_t c = 0; c < u.chunks.size(); ++c) pg_buffer_free_async(ctx, st, u.chunks[c]);
	}
	u.chunks.clear();
	u.used.clear();
}

void InputSide::clear()
{
	for (size_t t = 0; t < staged_.size(); ++t) release((int) t);
	host_.clear();
	staged_.clear();
	spans_.clear();
}

// ---------------------------------------------------------------------------
// Joins.
// ---------------------------------------------------------------------------
namespace {
// Column pruning between adjacent GPU joins: a join child that keeps its
// output on the device produces only the columns its parent reads (the
// parent's join key on that side and its projected columns of that side);
// `key` and the references' column numbers are remapped to the narrowed rows.
void prune_join_child(Operator* child, int side, unsigned& key, std::vector<std::pair<int, unsigned> >& refs)
{
	GpuJoinBase* cj = dynamic_cast<GpuJoinBase*>(child);
	if (!cj) return;
	const unsigned ncols = child->getOutSchema().columns();
	std::vector<bool> used(ncols, false);
	used[key] = true;
	for (size_t i = 0; i < refs.size(); ++i)
		if (refs[i].first == side) used[refs[i].second] = true;
	std::vector<unsigned> keep, remap(ncols, 0);
	for (unsigned i = 0; i < ncols; ++i)
		if (used[i]) { remap[i] = (unsigned) keep.size(); keep.push_back(i); }
	if (keep.size() == ncols) return;
	cj->narrow_projection(keep);
	key = remap[key];
	for (size_t i = 0; i < refs.size(); ++i)
		if (refs[i].first == side) refs[i].second = remap[refs[i].second];
}
}  // namespace

void GpuJoinBase::init(libconfig::Config& root, libconfig::Setting& node)
{
	Operator::init(root, node);
	libconfig::Setting& pr = node["projection"];
	// (side, column) of every output column: side 0 build, 1 probe.
	std::vector<std::pair<int, unsigned> > refs;
	for (int i = 0; i < pr.getLength(); ++i) {
		// "B$i" / "P$i" as createProjectionVector reads them (join.cpp:141-182).
		std::string s = pr[i];
		const std::string::size_type d = s.find('$');
		if (d == std::string::npos || d == 0) throw std::invalid_argument("bad projection `" + s + "'");
		std::istringstream is(s.substr(d + 1));
		unsigned attr = 0;
		is >> attr;
		if (!is) throw std::invalid_argument("bad projection `" + s + "'");
		const char side = s[d - 1];
		if (side != 'B' && side != 'P') throw std::invalid_argument("bad projection `" + s + "'");
		Schema& src = side == 'B' ? buildOp->getOutSchema() : probeOp->getOutSchema();
		if (attr >= src.columns()) throw std::invalid_argument("projection column out of range `" + s + "'");
		refs.push_back(std::make_pair(side == 'B' ? 0 : 1, attr));
	}
	buildkey_ = (int) node["buildjattr"];
	probekey_ = (int) node["probejattr"];
	if (buildkey_ >= buildOp->getOutSchema().columns() || probekey_ >= probeOp->getOutSchema().columns())
		throw std::invalid_argument("join attribute out of range");
	if (g_exchange) {
		prune_join_child(buildOp, 0, buildkey_, refs);
		prune_join_child(probeOp, 1, probekey_, refs);
	}
	Schema& bs = buildOp->getOutSchema();
	Schema& ps = probeOp->getOutSchema();
	for (size_t i = 0; i < refs.size(); ++i) {
		Schema& src = refs[i].first == 0 ? bs : ps;
		const unsigned attr = refs[i].second;
		schema.add(src.get(attr));
		pg_col c;
		c.side = refs[i].first == 0 ? 0 : 1;
		c.off = col_offset(src, attr);
		c.bytes = src.getColumnWidth(attr);
		cols_.push_back(c);
	}
	if (!key_bytes(bs, buildkey_) || key_bytes(bs, buildkey_) != key_bytes(ps, probekey_))
		throw std::invalid_argument("GPU joins need integer join keys of the same width on both sides");
	groups_.parse(node, 1);
	barriers_.clear();
	for (size_t g = 0; g < groups_.members.size(); ++g) {
		barriers_.push_back(new GroupBarrier());
		barriers_.back()->init((unsigned) groups_.members[g].size());
	}
	probe_filter_ = g_exchange ? dynamic_cast<GpuFilterOp*>(probeOp) : 0;
	probe_preds_.clear();
	if (probe_filter_) {
		probe_filter_->fuse_into_parent();
		probe_preds_ = probe_filter_->predicates();
	}
	node_ = node.getName() ? node.getName() : "";
	build_.setup(buildOp, node_);
	probe_.setup(probeOp, node_);
	group_rc_.assign(groups_.members.size(), PG_OK);
	output_.setup(groups_, schema.getTupleSize(), buffsize);
}

void GpuJoinBase::threadInit(unsigned short threadid)
{
	if (groups_.group_of.at(threadid) < 0) throw std::invalid_argument("thread not in any thread group");
}

pg_rel GpuJoinBase::side_rel(Operator* child, unsigned attr, const void* data, unsigned long long rows)
{
	Schema& s = child->getOutSchema();
	pg_rel r;
	r.width = s.getTupleSize();
	r.n = rows;
	r.data = rows ? data : 0;
	r.key_off = col_offset(s, attr);
	r.key_bytes = key_bytes(s, attr);
	return r;
}

// One launch over the group's inputs (staged uploads or a GPU child's device
// output); the rows are downloaded into the group's pages, or stay on the
// device for a GPU parent.
int GpuJoinBase::run_group(int g)
{
	const std::vector<int>& mem = groups_.members[g];
	const unsigned ow = schema.getTupleSize();
	pg_ctx* ctx = shared_context();
	if (!ctx) return PG_ERR_CUDA;
	const pg_stream st = thread_stream(ctx, mem[0]);
	int rc = PG_OK;
	const char *dR = 0, *dS = 0;
	unsigned long long nR = 0, nS = 0;
	void *tR = 0, *tS = 0, *dO = 0;
	unsigned long long rows = 0;
	const unsigned wR = buildOp->getOutSchema().getTupleSize(), wS = probeOp->getOutSchema().getTupleSize();
	void* tF = 0;
	// A probe side of several device arrays whose tuples are not 16 bytes is
	// probed array by array (the kernels for those widths append through one
	// output cursor), not copied together first; 16-byte tuples keep the
	// copy, for the positional kernel that needs one array.
	bool spans = false;
	if (!(rc = build_.gather(ctx, st, mem, wR, &dR, &nR, &tR)) && probe_preds_.empty() && wS != 16) {
		std::vector<std::pair<const char*, unsigned long long> > pcs;
		if (probe_.pieces(mem, wS, pcs) && pcs.size() > 1) {
			std::vector<pg_rel> srels;
			for (size_t i = 0; i < pcs.size(); ++i) srels.push_back(side_rel(probeOp, probekey_, pcs[i].first, pcs[i].second));
			trace(node_, mem[0], "gathered");
			const pg_rel r = side_rel(buildOp, buildkey_, dR, nR);
			rc = run_device_spans(ctx, st, r, srels, &dO, &rows);
			spans = rc != PG_ERR_UNSUPPORTED;
			if (!spans) rc = PG_OK;
			else trace(node_, mem[0], "joined");
		}
	}
	if (!rc && !spans && !(rc = probe_.gather(ctx, st, mem, wS, &dS, &nS, &tS))) {
		trace(node_, mem[0], "gathered");
		if (!probe_preds_.empty() && !probe_predicates() && nS) {
			// A fused gpufilter's predicates, applied to the probe side here.
			const pg_rel all = side_rel(probeOp, probekey_, dS, nS);
			uint64_t m = 0;
			if (!(rc = pg_buffer_alloc_async(ctx, st, nS * wS, &tF)) &&
					!(rc = pg_filter(ctx, st, &all, &probe_preds_[0], (int) probe_preds_.size(), tF, &m))) {
				dS = (const char*) tF;
				nS = m;
			}
		}
		const pg_rel r = side_rel(buildOp, buildkey_, dR, nR);
		const pg_rel s = side_rel(probeOp, probekey_, dS, nS);
		if (!rc) rc = run_device(ctx, st, r, s, &dO, &rows);
		trace(node_, mem[0], "joined");
	}
	if (!rc && !on_device_) {
		std::vector<char>& out = output_.buffer(g);
		out.resize((size_t) (rows * ow));
		if (rows) rc = pg_d2h(ctx, st, &out[0], dO, rows * ow);
		if (!rc) count(&g_stats.d2h, rows * ow);
	}
	for (size_t i = 0; i < mem.size(); ++i) { build_.release(mem[i], st); probe_.release(mem[i], st); }
	if (tR) pg_buffer_free_async(ctx, st, tR);
	if (tS) pg_buffer_free_async(ctx, st, tS);
	if (tF) pg_buffer_free_async(ctx, st, tF);
	if (!rc) rc = pg_sync(ctx, st);
	if (!rc && on_device_) {
		output_.set_device(g, (const char*) dO, rows);
		if (dO) output_.own_device(dO);
		dO = 0;
	} else {
		output_.set_rows(g, rc ? 0 : rows);
	}
	if (dO) pg_buffer_free_async(ctx, st, dO);
	return rc;
}

Operator::ResultCode GpuJoinBase::scanStart(unsigned short tid, Page* idx, Schema& idxs)
{
	const int g = groups_.group_of[tid];
	trace(node_, tid, "start");
	ResultCode rc = buildOp->scanStart(tid, idx, idxs);
	bool ok = rc != Error && build_.fetch(buildOp, tid);
	if (probeOp->scanStart(tid, idx, idxs) == Error) ok = false;
	ok = ok && probe_.fetch(probeOp, tid);
	if (!ok) group_rc_[g] = PG_ERR_ARG;
	barriers_[g]->arrive();
	const std::vector<int>& mem = groups_.members[g];
	if (tid == mem[0] && group_rc_[g] == PG_OK) {
		trace(node_, tid, "launch");
		group_rc_[g] = run_group(g);
		trace(node_, tid, "done");
		if (group_rc_[g] != PG_OK) note_failure("gpu join", group_rc_[g]);
	}
	barriers_[g]->arrive();
	if (group_rc_[g] != PG_OK) return Error;
	output_.assign(tid, g, groups_.pos_in[tid], (int) mem.size());
	return Ready;
}

void GpuJoinBase::narrow_projection(const std::vector<unsigned>& keep)
{
	std::vector<pg_col> cols;
	Schema narrowed;
	for (size_t i = 0; i < keep.size(); ++i) {
		cols.push_back(cols_.at(keep[i]));
		narrowed.add(schema.get(keep[i]));
	}
	cols_ = cols;
	schema = narrowed;
	output_.setup(groups_, schema.getTupleSize(), buffsize);
}

Operator::GetNextResultT GpuJoinBase::getNext(unsigned short tid)
{
	if (on_device_ || group_rc_[groups_.group_of[tid]] != PG_OK) return std::make_pair(Error, (Page*) 0);
	return output_.next(tid);
}

Operator::ResultCode GpuJoinBase::scanStop(unsigned short tid)
{
	return DualInputOp::scanStop(tid);
}

void GpuJoinBase::threadClose(unsigned short tid)
{
	(void) tid;     // inputs are released by the group's launch
}

void GpuJoinBase::destroy()
{
	output_.clear();
	for (size_t g = 0; g < barriers_.size(); ++g) delete barriers_[g];
	barriers_.clear();
}

int GpuHashJoinOp::run_device(pg_ctx* ctx, pg_stream st, const pg_rel& R, const pg_rel& S, void** out,
		unsigned long long* rows)
{
	const unsigned ow = schema.getTupleSize();
	pg_hashtable* ht = 0;
	int rc = pg_hashjoin_build(ctx, st, &R, &cols_[0], (int) cols_.size(), &ht);
	if (rc) return rc;
	trace(node_, 0, "built");
	unsigned long long cap = std::max<unsigned long long>(S.n, 1);
	void* o = 0;
	pg_join_result res;
	res.n_out = 0; res.sum = 0;
	for (int attempt = 0; attempt < 2; ++attempt) {
		if ((rc = pg_buffer_alloc_async(ctx, st, cap * ow, &o))) break;
		trace(node_, 0, "out allocated");
		rc = pg_hashjoin_probe_where(ctx, st, ht, &S, probe_preds_.empty() ? 0 : &probe_preds_[0],
				(int) probe_preds_.size(), &cols_[0], (int) cols_.size(), o, cap, PG_JOIN_MATERIALIZE, -1, &res);
		if (rc == PG_ERR_OUTPUT_FULL && attempt == 0) {
			pg_buffer_free_async(ctx, st, o);
			o = 0;
			cap = res.n_out;
			continue;
		}
		break;
	}
	pg_hashtable_free(ctx, ht);
	if (rc) { if (o) pg_buffer_free_async(ctx, st, o); return rc; }
	*out = o;
	*rows = res.n_out;
	return PG_OK;
}

int GpuHashJoinOp::run_device_spans(pg_ctx* ctx, pg_stream st, const pg_rel& R, const std::vector<pg_rel>& S,
		void** out, unsigned long long* rows)
{
	const unsigned ow = schema.getTupleSize();
	pg_hashtable* ht = 0;
	int rc = pg_hashjoin_build(ctx, st, &R, &cols_[0], (int) cols_.size(), &ht);
	if (rc) return rc;
	trace(node_, 0, "built");
	unsigned long long cap = 0;
	for (size_t i = 0; i < S.size(); ++i) cap += S[i].n;
	cap = std::max<unsigned long long>(cap, 1);
	void* o = 0;
	pg_join_result res;
	res.n_out = 0; res.sum = 0;
	for (int attempt = 0; attempt < 2; ++attempt) {
		if ((rc = pg_buffer_alloc_async(ctx, st, cap * ow, &o))) break;
		rc = pg_hashjoin_probe_spans(ctx, st, ht, &S[0], (int) S.size(), &cols_[0], (int) cols_.size(), o, cap,
				PG_JOIN_MATERIALIZE, -1, &res);
		if (rc == PG_ERR_OUTPUT_FULL && attempt == 0) {
			pg_buffer_free_async(ctx, st, o);
			o = 0;
			cap = res.n_out;
			continue;
		}
		break;
	}
	pg_hashtable_free(ctx, ht);
	if (rc) { if (o) pg_buffer_free_async(ctx, st, o); return rc; }
	*out = o;
	*rows = res.n_out;
	return PG_OK;
}

void GpuMPSMJoinOp::init(libconfig::Config& root, libconfig::Setting& node)
{
	GpuJoinBase::init(root, node);
	std::string v;
	sorted_flags_ = 0;
	if (node.lookupValue("buildpresorted", v) && v == "yes") sorted_flags_ |= PG_JOIN_BUILD_SORTED;
	if (node.lookupValue("probepresorted", v) && v == "yes") sorted_flags_ |= PG_JOIN_PROBE_SORTED;
}

int GpuMPSMJoinOp::run_device(pg_ctx* ctx, pg_stream st, const pg_rel& R, const pg_rel& S, void** out,
		unsigned long long* rows)
{
	const unsigned ow = schema.getTupleSize();
	pg_join_result res;
	res.n_out = 0; res.sum = 0;
	// Room for |R| + |S| rows first (a PK-FK join's output); a join that needs
	// more reports its size and runs again into a buffer of exactly that.
	unsigned long long cap = std::max<unsigned long long>(R.n + S.n, 1);
	for (int attempt = 0; attempt < 2; ++attempt) {
		void* o = 0;
		int rc = pg_buffer_alloc_async(ctx, st, cap * ow, &o);
		if (rc) return rc;
		rc = pg_mpsm_join(ctx, st, &R, &S, &cols_[0], (int) cols_.size(), o, cap,
				PG_JOIN_MATERIALIZE | sorted_flags_, -1, &res);
		if (rc == PG_OK) {
			*out = o;
			*rows = res.n_out;
			return PG_OK;
		}
		pg_buffer_free_async(ctx, st, o);
		if (rc != PG_ERR_OUTPUT_FULL || attempt) return rc;
		cap = std::max<unsigned long long>(res.n_out, 1);
	}
	return PG_ERR_OUTPUT_FULL;
}

// ---------------------------------------------------------------------------
// Partition.
// ---------------------------------------------------------------------------
void GpuPartitionOp::init(libconfig::Config& root, libconfig::Setting& node)
{
	Operator::init(root, node);
	schema = nextOp->getOutSchema();
	attr_ = (int) node["attr"];
	if (attr_ >= schema.columns() || !key_bytes(schema, attr_))
		throw std::invalid_argument("gpupartition: attr must be an integer column");
	std::string fn = "exactrange";
	node.lookupValue("fn", fn);
	memset(&cfg_, 0, sizeof cfg_);
	cfg_.fn = hash_fn_code(fn);
	cfg_.buckets = (int) node["buckets"];
	if (cfg_.fn == PG_FN_EXACTRANGE || cfg_.fn == PG_FN_RANGE) {
		cfg_.min = (long) node["range"][0];
		cfg_.max = (long) node["range"][1];
	}
	node.lookupValue("skipbits", cfg_.skipbits);
	node.lookupValue("offset", cfg_.offset);
	pg_ctx* ctx = shared_context();
	uint32_t nb = cfg_.buckets;
	if (ctx && pg_hash_buckets(ctx, &cfg_, &nb) != PG_OK)
		throw std::invalid_argument("gpupartition: unsupported hash configuration");
	nparts_ = nb;
	if (nparts_ < 1 || nparts_ >= MAX_THREADS) throw std::invalid_argument("gpupartition: one thread per partition");
	std::string s;
	sort_ = node.lookupValue("sort", s) && s == "yes";
	sortattr_ = attr_;
	if (sort_) node.lookupValue("sortattr", sortattr_);
	if (sort_ && (sortattr_ >= schema.columns() || !key_bytes(schema, sortattr_)))
		throw std::invalid_argument("gpupartition: sortattr must be an integer column");
	barrier_.init(nparts_);
	node_ = node.getName() ? node.getName() : "";
	in_.setup(nextOp, node_);
	rc_ = PG_OK;
	// One group of nparts_ threads; partition t is served whole by thread t.
	one_group_.group_of.assign(MAX_THREADS, -1);
	one_group_.pos_in.assign(MAX_THREADS, -1);
	one_group_.members.assign(nparts_, std::vector<int>());
	for (unsigned t = 0; t < nparts_; ++t) {
		one_group_.group_of[t] = (int) t;
		one_group_.pos_in[t] = 0;
		one_group_.members[t].push_back((int) t);
	}
	served_.setup(one_group_, schema.getTupleSize(), buffsize);
}

void GpuPartitionOp::threadInit(unsigned short tid)
{
	if (tid >= nparts_) throw std::invalid_argument("gpupartition: more threads than partitions");
}

// One launch over all threads' input (thread order); partition t goes to
// thread t, downloaded into its pages or left on the device for a GPU parent.
int GpuPartitionOp::run_partition()
{
	const unsigned w = schema.getTupleSize();
	pg_ctx* ctx = shared_context();
	if (!ctx) return PG_ERR_CUDA;
	std::vector<int> all(nparts_);
	for (unsigned t = 0; t < nparts_; ++t) all[t] = (int) t;
	const pg_stream st = thread_stream(ctx, 0);
	int rc = PG_OK;
	const char* din = 0;
	unsigned long long n = 0;
	void *tin = 0, *dout = 0, *doffs = 0, *scratch = 0;
	offsets_.assign(nparts_ + 1, 0);
	if (!rc) rc = in_.gather(ctx, st, all, w, &din, &n, &tin);
	if (!rc) rc = pg_buffer_alloc_async(ctx, st, n ? n * w : 16, &dout);
	if (!rc) rc = pg_buffer_alloc_async(ctx, st, (nparts_ + 1) * 8, &doffs);
	pg_rel r;
	r.data = din; r.n = n; r.width = w;
	r.key_off = col_offset(schema, attr_); r.key_bytes = key_bytes(schema, attr_);
	if (!rc) rc = pg_partition(ctx, st, &r, &cfg_, dout, (uint64_t*) doffs);
	if (!rc) rc = pg_d2h(ctx, st, &offsets_[0], doffs, (nparts_ + 1) * 8);
	if (!rc) rc = pg_sync(ctx, st);
	if (!rc && sort_ && n) {
		pg_rel p = r;
		p.data = dout;
		p.key_off = col_offset(schema, sortattr_); p.key_bytes = key_bytes(schema, sortattr_);
		// The input may be the child's output: sort with scratch of our own.
		if (tin) scratch = tin;
		else if (!(rc = pg_buffer_alloc_async(ctx, st, n * w, &tin))) scratch = tin;
		if (!rc) rc = pg_partition_sort(ctx, st, &p, &offsets_[0], nparts_, scratch);
	}
	for (unsigned t = 0; t < nparts_ && !rc; ++t) {
		const unsigned long long rows = offsets_[t + 1] - offsets_[t];
		if (on_device_) {
			served_.set_device((int) t, (const char*) dout + offsets_[t] * w, rows);
			continue;
		}
		std::vector<char>& o = served_.buffer((int) t);
		o.resize((size_t) (rows * w));
		if (rows) rc = pg_d2h(ctx, st, &o[0], (char*) dout + offsets_[t] * w, rows * w);
		count(&g_stats.d2h, rows * w);
		served_.set_rows((int) t, rows);
	}
	for (unsigned t = 0; t < nparts_; ++t) in_.release((int) t, st);
	if (tin) pg_buffer_free_async(ctx, st, tin);
	if (!rc) rc = pg_sync(ctx, st);
	if (!rc && on_device_) { served_.own_device(dout); dout = 0; }
	if (doffs) pg_buffer_free_async(ctx, st, doffs);
	if (dout) pg_buffer_free_async(ctx, st, dout);
	return rc;
}

Operator::ResultCode GpuPartitionOp::scanStart(unsigned short tid, Page* idx, Schema& idxs)
{
	bool ok = nextOp->scanStart(tid, idx, idxs) != Error && in_.fetch(nextOp, tid);
	if (!ok) rc_ = PG_ERR_ARG;
	barrier_.arrive();
	if (tid == 0 && rc_ == PG_OK) {
		rc_ = run_partition();
		if (rc_) note_failure("gpupartition", rc_);
	}
	barrier_.arrive();
	if (rc_ != PG_OK) return Error;
	served_.assign(tid, (int) tid, 0, 1);
	return Ready;
}

Operator::GetNextResultT GpuPartitionOp::getNext(unsigned short tid)
{
	if (on_device_ || rc_ != PG_OK) return std::make_pair(Error, (Page*) 0);
	return served_.next(tid);
}

Operator::ResultCode GpuPartitionOp::scanStop(unsigned short tid)
{
	return nextOp->scanStop(tid);
}

void GpuPartitionOp::destroy()
{
	served_.clear();
}

// ---------------------------------------------------------------------------
// Aggregates.
// ---------------------------------------------------------------------------
void GpuAggregateOp::init(libconfig::Config& root, libconfig::Setting& node)
{
	Operator::init(root, node);
	Schema& in = nextOp->getOutSchema();
	if (node.exists("fields")) {
		libconfig::Setting& f = node["fields"];
		if (f.getLength() > 1) throw std::invalid_argument("GPU aggregates group by one column");
		field_ = f.getLength() ? (int) f[0] : -1;
	} else {
		field_ = (int) node["field"];
	}
	if (field_ >= 0 && ((unsigned) field_ >= in.columns() || !key_bytes(in, field_)))
		throw std::invalid_argument("GPU aggregates group by an integer column");
	if (field_ >= 0) schema.add(in.get(field_));
	if (agg_ == PG_AGG_SUM) {
		sumfield_ = (int) node["sumfield"];
		if (sumfield_ >= in.columns()) throw std::invalid_argument("sumfield out of range");
		const ColumnType t = in.getColumnType(sumfield_);
		if (t != CT_INTEGER && t != CT_LONG && t != CT_DECIMAL)
			throw std::invalid_argument("sumfield must be int, long or dec");
		schema.add(t);
	} else {
		schema.add(CT_LONG);
	}
	global_ = node.exists("global");
	threads_ = 1;
	if (global_) threads_ = (int) node["threads"];
	if (threads_ < 1 || threads_ > MAX_THREADS) throw std::invalid_argument("threads out of range");
	groups_.group_of.assign(MAX_THREADS, -1);
	groups_.pos_in.assign(MAX_THREADS, -1);
	groups_.members.clear();
	if (global_) {
		groups_.members.push_back(std::vector<int>());
		for (unsigned t = 0; t < threads_; ++t) { groups_.group_of[t] = 0; groups_.pos_in[t] = (int) t; groups_.members[0].push_back((int) t); }
	} else {
		// Thread-local: every thread is a group of its own.
		for (int t = 0; t < MAX_THREADS; ++t) {
			groups_.group_of[t] = t; groups_.pos_in[t] = 0;
			groups_.members.push_back(std::vector<int>(1, t));
		}
	}
	barrier_.init(threads_);
	node_ = node.getName() ? node.getName() : "";
	in_.setup(nextOp, node_);
	rc_ = PG_OK;
	output_.setup(groups_, schema.getTupleSize(), buffsize);
}

void GpuAggregateOp::threadInit(unsigned short tid)
{
	if (global_ && tid >= threads_) throw std::invalid_argument("thread id beyond `threads'");
}

int GpuAggregateOp::aggregate(const std::vector<int>& members, int g)
{
	pg_ctx* ctx = shared_context();
	if (!ctx) return PG_ERR_CUDA;
	Schema& is = nextOp->getOutSchema();
	const unsigned w = is.getTupleSize(), ow = schema.getTupleSize();
	const pg_stream st = thread_stream(ctx, members[0]);
	int rc = PG_OK;
	const char* din = 0;
	unsigned long long n = 0;
	void *tin = 0, *dout = 0;
	uint64_t ng = 0;
	// Output room for up to 1M groups first (at most one per input row); a
	// larger count is reported by pg_groupby and the aggregation reruns with
	// room for exactly that many.
	unsigned long long cap = 1;
	if (!(rc = in_.gather(ctx, st, members, w, &din, &n, &tin)))
		cap = std::max<unsigned long long>(1, std::min<unsigned long long>(n, 1ull << 20));
	if (!rc && !(rc = pg_buffer_alloc_async(ctx, st, cap * ow, &dout))) {
		trace(node_, members[0], "gathered");
		pg_rel r;
		r.data = din; r.n = n; r.width = w;
		r.key_off = field_ >= 0 ? col_offset(is, field_) : 0;
		r.key_bytes = field_ >= 0 ? key_bytes(is, field_) : 0;
		const unsigned voff = agg_ == PG_AGG_SUM ? col_offset(is, sumfield_) : 0;
		int vt = PG_VAL_LONG;
		if (agg_ == PG_AGG_SUM) {
			const ColumnType t = is.getColumnType(sumfield_);
			vt = t == CT_INTEGER ? PG_VAL_INT : t == CT_DECIMAL ? PG_VAL_DEC : PG_VAL_LONG;
		}
		rc = pg_groupby(ctx, st, &r, voff, vt, agg_, 0, dout, cap, &ng);
		if (rc == PG_ERR_OUTPUT_FULL) {
			pg_buffer_free_async(ctx, st, dout);
			dout = 0;
			cap = ng;
			if (!(rc = pg_buffer_alloc_async(ctx, st, cap * ow, &dout)))
				rc = pg_groupby(ctx, st, &r, voff, vt, agg_, 0, dout, cap, &ng);
		}
		if (!rc && !on_device_) {
			std::vector<char>& out = output_.buffer(g);
			out.resize((size_t) (ng * ow));
			if (ng) rc = pg_d2h(ctx, st, &out[0], dout, ng * ow);
			count(&g_stats.d2h, ng * ow);
		}
	}
	for (size_t i = 0; i < members.size(); ++i) in_.release(members[i], st);
	if (tin) pg_buffer_free_async(ctx, st, tin);
	if (!rc) rc = pg_sync(ctx, st);
	if (!rc && on_device_) {
		output_.set_device(g, (const char*) dout, ng);
		output_.own_device(dout);
		dout = 0;
	} else {
		output_.set_rows(g, rc ? 0 : ng);
	}
	if (dout) pg_buffer_free_async(ctx, st, dout);
	return rc;
}

Operator::ResultCode GpuAggregateOp::scanStart(unsigned short tid, Page* idx, Schema& idxs)
{
	trace(node_, tid, "start");
	bool ok = nextOp->scanStart(tid, idx, idxs) != Error && in_.fetch(nextOp, tid);
	// The scan of the input ends inside scanStart, as GenericAggregate's does.
	if (nextOp->scanStop(tid) == Error) ok = false;
	if (!global_) {
		int rc = ok ? aggregate(std::vector<int>(1, (int) tid), tid) : PG_ERR_ARG;
		if (rc) { note_failure("gpuaggregate", rc); return Error; }
		output_.assign(tid, tid, 0, 1);
		return Ready;
	}
	if (!ok) rc_ = PG_ERR_ARG;
	barrier_.arrive();
	if (tid == 0 && rc_ == PG_OK) {
		trace(node_, tid, "launch");
		rc_ = aggregate(groups_.members[0], 0);
		trace(node_, tid, "done");
		if (rc_) note_failure("gpuaggregate", rc_);
	}
	barrier_.arrive();
	if (rc_ != PG_OK) return Error;
	output_.assign(tid, 0, (int) tid, (int) threads_);
	return Ready;
}

Operator::GetNextResultT GpuAggregateOp::getNext(unsigned short tid)
{
	if (on_device_ || (global_ && rc_ != PG_OK)) return std::make_pair(Error, (Page*) 0);
	return output_.next(tid);
}

Operator::ResultCode GpuAggregateOp::scanStop(unsigned short tid)
{
	(void) tid;
	return Ready;   // the input scan was stopped in scanStart
}

void GpuAggregateOp::destroy()
{
	output_.clear();
}

// ---------------------------------------------------------------------------
// Filter and Project.
// ---------------------------------------------------------------------------
namespace {
// Comparator::parseString (comparator.cpp:415-431).
uint32_t cmp_code(const std::string& op)
{
	if (op == "<") return PG_CMP_LT;
	if (op == "<=") return PG_CMP_LE;
	if (op == "=" || op == "==") return PG_CMP_EQ;
	if (op == "<>" || op == "!=") return PG_CMP_NE;
	if (op == ">=") return PG_CMP_GE;
	if (op == ">") return PG_CMP_GT;
	throw std::invalid_argument("gpufilter: unknown comparison `" + op + "'");
}

// Per-thread groups: every thread a group of its own.
void one_group_per_thread(ThreadGroups& g)
{
	g.group_of.assign(MAX_THREADS, -1);
	g.pos_in.assign(MAX_THREADS, -1);
	g.members.clear();
	for (int t = 0; t < MAX_THREADS; ++t) {
		g.group_of[t] = t; g.pos_in[t] = 0;
		g.members.push_back(std::vector<int>(1, t));
	}
}
}  // namespace

void GpuFilterOp::init(libconfig::Config& root, libconfig::Setting& node)
{
	Operator::init(root, node);
	schema = nextOp->getOutSchema();
	const unsigned field = (int) node["field"];
	if (field >= schema.columns()) throw std::invalid_argument("gpufilter: field out of range");
	std::string op = node["op"];
	std::string value = node["value"];
	pg_pred p;
	memset(&p, 0, sizeof p);
	p.op = cmp_code(op);
	p.off = col_offset(schema, field);
	p.bytes = schema.getColumnWidth(field);
	switch (schema.getColumnType(field)) {
	case CT_INTEGER: p.type = PG_PRED_INT; break;
	case CT_LONG: case CT_DATE: p.type = PG_PRED_LONG; break;
	case CT_DECIMAL: p.type = PG_PRED_DEC; break;
	case CT_CHAR: p.type = PG_PRED_CHAR; break;
	default: throw std::invalid_argument("gpufilter: unsupported column type");
	}
	if (p.bytes > sizeof p.value) throw std::invalid_argument("gpufilter: column wider than 128 bytes");
	// The constant in the column's own form, parsed as Filter parses it
	// (filter.cpp:57-64): a one-column schema of the same column.
	Schema one;
	one.add(schema.get(field));
	const char* text = value.c_str();
	one.parseTuple(p.value, &text);
	preds_.clear();
	preds_.push_back(p);
	// A gpufilter right below hands its input up: both predicates in one pass.
	GpuFilterOp* below = g_exchange ? dynamic_cast<GpuFilterOp*>(nextOp) : 0;
	if (below) {
		below->fuse_into_parent();
		const std::vector<pg_pred>& more = below->predicates();
		preds_.insert(preds_.end(), more.begin(), more.end());
		if (preds_.size() > PG_PRED_MAX) throw std::invalid_argument("gpufilter: at most 4 filters in a row");
	}
	node_ = node.getName() ? node.getName() : "";
	in_.setup(nextOp, node_);
	one_group_per_thread(groups_);
	output_.setup(groups_, schema.getTupleSize(), buffsize);
	rc_.assign(MAX_THREADS, PG_OK);
}

void GpuFilterOp::threadInit(unsigned short tid)
{
	(void) tid;
}

// This thread's input, filtered (or, fused, handed through unfiltered).
int GpuFilterOp::run(unsigned short tid)
{
	pg_ctx* ctx = shared_context();
	if (!ctx) return PG_ERR_CUDA;
	const unsigned w = schema.getTupleSize();
	const pg_stream st = thread_stream(ctx, tid);
	int rc = PG_OK;
	const char* din = 0;
	unsigned long long n = 0;
	void *tin = 0, *dout = 0;
	uint64_t m = 0;
	rc = in_.gather(ctx, st, std::vector<int>(1, (int) tid), w, &din, &n, &tin);
	if (!rc && fused_) {
		// The parent applies the predicates; the input stays as it is (its
		// staged memory lives until destroy).
		if (!(rc = pg_sync(ctx, st))) {
			output_.set_device(tid, din, n);
			if (tin) output_.own_device(tin);
			tin = 0;
		}
	} else if (!rc) {
		pg_rel r;
		r.data = din; r.n = n; r.width = w; r.key_off = 0; r.key_bytes = 0;
		if (!(rc = pg_buffer_alloc_async(ctx, st, std::max<unsigned long long>(n, 1) * w, &dout)) &&
				!(rc = pg_filter(ctx, st, &r, &preds_[0], (int) preds_.size(), dout, &m))) {
			if (on_device_) {
				output_.set_device(tid, (const char*) dout, m);
				output_.own_device(dout);
				dout = 0;
			} else {
				std::vector<char>& out = output_.buffer(tid);
				out.resize((size_t) (m * w));
				if (m) rc = pg_d2h(ctx, st, &out[0], dout, m * w);
				count(&g_stats.d2h, m * w);
				output_.set_rows(tid, rc ? 0 : m);
			}
		}
		in_.release(tid, st);
		if (tin) pg_buffer_free_async(ctx, st, tin);
		if (!rc) rc = pg_sync(ctx, st);
	}
	if (dout) pg_buffer_free_async(ctx, st, dout);
	return rc;
}

Operator::ResultCode GpuFilterOp::scanStart(unsigned short tid, Page* idx, Schema& idxs)
{
	bool ok = nextOp->scanStart(tid, idx, idxs) != Error && in_.fetch(nextOp, tid);
	int rc = ok ? run(tid) : PG_ERR_ARG;
	rc_[tid] = rc;
	if (rc) { note_failure("gpufilter", rc); return Error; }
	output_.assign(tid, tid, 0, 1);
	return Ready;
}

Operator::GetNextResultT GpuFilterOp::getNext(unsigned short tid)
{
	if (on_device_ || rc_[tid] != PG_OK) return std::make_pair(Error, (Page*) 0);
	return output_.next(tid);
}

Operator::ResultCode GpuFilterOp::scanStop(unsigned short tid)
{
	return nextOp->scanStop(tid);
}

void GpuFilterOp::destroy()
{
	output_.clear();
	in_.clear();
}

void GpuProjectOp::init(libconfig::Config& root, libconfig::Setting& node)
{
	Operator::init(root, node);
	Schema& src = nextOp->getOutSchema();
	libconfig::Setting& pr = node["projection"];
	proj_.clear();
	cols_.clear();
	for (int i = 0; i < pr.getLength(); ++i) {
		// "$i" as Project's parseInput reads it (project.cpp:37-50).
		std::string s = pr[i];
		const std::string::size_type d = s.find('$');
		unsigned attr = 0;
		std::istringstream is(d == std::string::npos ? std::string() : s.substr(d + 1));
		is >> attr;
		if (d == std::string::npos || !is) throw std::invalid_argument("gpuproject: bad projection `" + s + "'");
		if (attr >= src.columns()) throw std::invalid_argument("gpuproject: projection column out of range");
		proj_.push_back(attr);
		pg_col c;
		c.side = 0;
		c.off = col_offset(src, attr);
		c.bytes = src.getColumnWidth(attr);
		cols_.push_back(c);
		schema.add(src.get(attr));
	}
	join_ = g_exchange ? dynamic_cast<GpuJoinBase*>(nextOp) : 0;
	if (join_) {
		join_->narrow_projection(proj_);
		return;
	}
	node_ = node.getName() ? node.getName() : "";
	in_.setup(nextOp, node_);
	one_group_per_thread(groups_);
	output_.setup(groups_, schema.getTupleSize(), buffsize);
	rc_.assign(MAX_THREADS, PG_OK);
}

void GpuProjectOp::threadInit(unsigned short tid)
{
	(void) tid;
}

void GpuProjectOp::keep_on_device()
{
	on_device_ = true;
	if (join_) join_->keep_on_device();
}

DeviceSpan GpuProjectOp::device_share(unsigned short tid)
{
	return join_ ? join_->device_share(tid) : output_.share(tid);
}

int GpuProjectOp::run(unsigned short tid)
{
	pg_ctx* ctx = shared_context();
	if (!ctx) return PG_ERR_CUDA;
	const unsigned w = nextOp->getOutSchema().getTupleSize(), ow = schema.getTupleSize();
	const pg_stream st = thread_stream(ctx, tid);
	int rc = PG_OK;
	const char* din = 0;
	unsigned long long n = 0;
	void *tin = 0, *dout = 0;
	if (!(rc = in_.gather(ctx, st, std::vector<int>(1, (int) tid), w, &din, &n, &tin)) &&
			!(rc = pg_buffer_alloc_async(ctx, st, std::max<unsigned long long>(n, 1) * ow, &dout))) {
		pg_rel r;
		r.data = din; r.n = n; r.width = w; r.key_off = 0; r.key_bytes = 0;
		if (!(rc = pg_project(ctx, st, &r, &cols_[0], (int) cols_.size(), dout))) {
			if (on_device_) {
				output_.set_device(tid, (const char*) dout, n);
				output_.own_device(dout);
				dout = 0;
			} else {
				std::vector<char>& out = output_.buffer(tid);
				out.resize((size_t) (n * ow));
				if (n) rc = pg_d2h(ctx, st, &out[0], dout, n * ow);
				count(&g_stats.d2h, n * ow);
				output_.set_rows(tid, rc ? 0 : n);
			}
		}
	}
	in_.release(tid, st);
	if (tin) pg_buffer_free_async(ctx, st, tin);
	if (!rc) rc = pg_sync(ctx, st);
	if (dout) pg_buffer_free_async(ctx, st, dout);
	return rc;
}

Operator::ResultCode GpuProjectOp::scanStart(unsigned short tid, Page* idx, Schema& idxs)
{
	if (join_) return nextOp->scanStart(tid, idx, idxs);
	bool ok = nextOp->scanStart(tid, idx, idxs) != Error && in_.fetch(nextOp, tid);
	int rc = ok ? run(tid) : PG_ERR_ARG;
	rc_[tid] = rc;
	if (rc) { note_failure("gpuproject", rc); return Error; }
	output_.assign(tid, tid, 0, 1);
	return Ready;
}

Operator::GetNextResultT GpuProjectOp::getNext(unsigned short tid)
{
	if (join_) return nextOp->getNext(tid);
	if (on_device_ || rc_[tid] != PG_OK) return std::make_pair(Error, (Page*) 0);
	return output_.next(tid);
}

Operator::ResultCode GpuProjectOp::scanStop(unsigned short tid)
{
	return nextOp->scanStop(tid);
}

void GpuProjectOp::destroy()
{
	output_.clear();
	in_.clear();
}

Operator* create(const std::string& type)
{
	if (type == "gpuhashjoin") return new GpuHashJoinOp();
	if (type == "gpumpsmjoin") return new GpuMPSMJoinOp();
	if (type == "gpupartition") return new GpuPartitionOp();
	if (type == "gpuaggregate_sum") return new GpuAggregateSumOp();
	if (type == "gpuaggregate_count") return new GpuAggregateCountOp();
	if (type == "gpufilter") return new GpuFilterOp();
	if (type == "gpuproject") return new GpuProjectOp();
	return 0;
}

}  // namespace pythia_gpu_ops
