// GPU operators for Pythia plans (see gpuops.h). C++98, like the engine.
#include "gpuops.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <sstream>
#include <stdexcept>

namespace pythia_gpu_ops {

// ---------------------------------------------------------------------------
// Context, failures, barrier, thread groups.
// ---------------------------------------------------------------------------
namespace {
pthread_once_t g_once = PTHREAD_ONCE_INIT;
pg_ctx* g_ctx = 0;
pthread_mutex_t g_fail_mu = PTHREAD_MUTEX_INITIALIZER;
std::string g_fail;

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
	Cursor c = { 0, 0, 0, true };
	cur_.assign(MAX_THREADS, c);
}

void GroupedOutput::assign(int tid, int group, int pos, int k)
{
	const unsigned long long rows = rows_[group];
	const unsigned long long lo = rows * pos / k, hi = rows * (pos + 1) / k;
	Cursor& c = cur_[tid];
	c.at = out_[group].empty() ? 0 : &out_[group][0] + lo * tuple_size_;
	c.left = (hi - lo) * tuple_size_;
	c.done = false;
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

// ---------------------------------------------------------------------------
// Joins.
// ---------------------------------------------------------------------------
void GpuJoinBase::init(libconfig::Config& root, libconfig::Setting& node)
{
	Operator::init(root, node);
	libconfig::Setting& pr = node["projection"];
	Schema& bs = buildOp->getOutSchema();
	Schema& ps = probeOp->getOutSchema();
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
		Schema& src = side == 'B' ? bs : ps;
		if (attr >= src.columns()) throw std::invalid_argument("projection column out of range `" + s + "'");
		schema.add(src.get(attr));
		pg_col c;
		c.side = side == 'B' ? 0 : 1;
		c.off = col_offset(src, attr);
		c.bytes = src.getColumnWidth(attr);
		cols_.push_back(c);
	}
	buildkey_ = (int) node["buildjattr"];
	probekey_ = (int) node["probejattr"];
	if (buildkey_ >= bs.columns() || probekey_ >= ps.columns())
		throw std::invalid_argument("join attribute out of range");
	if (!key_bytes(bs, buildkey_) || key_bytes(bs, buildkey_) != key_bytes(ps, probekey_))
		throw std::invalid_argument("GPU joins need integer join keys of the same width on both sides");
	groups_.parse(node, 1);
	barriers_.clear();
	for (size_t g = 0; g < groups_.members.size(); ++g) {
		barriers_.push_back(new GroupBarrier());
		barriers_.back()->init((unsigned) groups_.members[g].size());
	}
	build_in_.assign(MAX_THREADS, std::vector<char>());
	probe_in_.assign(MAX_THREADS, std::vector<char>());
	group_rc_.assign(groups_.members.size(), PG_OK);
	output_.setup(groups_, schema.getTupleSize(), buffsize);
}

void GpuJoinBase::threadInit(unsigned short threadid)
{
	if (groups_.group_of.at(threadid) < 0) throw std::invalid_argument("thread not in any thread group");
}

pg_rel GpuJoinBase::side_rel(Operator* child, unsigned attr, const std::vector<char>& data)
{
	Schema& s = child->getOutSchema();
	pg_rel r;
	r.width = s.getTupleSize();
	r.n = r.width ? data.size() / r.width : 0;
	r.data = data.empty() ? 0 : &data[0];
	r.key_off = col_offset(s, attr);
	r.key_bytes = key_bytes(s, attr);
	return r;
}

Operator::ResultCode GpuJoinBase::scanStart(unsigned short tid, Page* idx, Schema& idxs)
{
	const int g = groups_.group_of[tid];
	ResultCode rc = buildOp->scanStart(tid, idx, idxs);
	bool ok = rc != Error && drain(buildOp, tid, build_in_[tid]);
	if (probeOp->scanStart(tid, idx, idxs) == Error) ok = false;
	ok = ok && drain(probeOp, tid, probe_in_[tid]);
	if (!ok) group_rc_[g] = PG_ERR_ARG;
	barriers_[g]->arrive();
	const std::vector<int>& mem = groups_.members[g];
	if (tid == mem[0] && group_rc_[g] == PG_OK) {
		std::vector<char> R, S;
		for (size_t i = 0; i < mem.size(); ++i) {
			R.insert(R.end(), build_in_[mem[i]].begin(), build_in_[mem[i]].end());
			S.insert(S.end(), probe_in_[mem[i]].begin(), probe_in_[mem[i]].end());
			std::vector<char>().swap(build_in_[mem[i]]);
			std::vector<char>().swap(probe_in_[mem[i]]);
		}
		unsigned long long rows = 0;
		const pg_rel r = side_rel(buildOp, buildkey_, R), s = side_rel(probeOp, probekey_, S);
		group_rc_[g] = run_group(r, s, output_.buffer(g), &rows);
		if (group_rc_[g] != PG_OK) note_failure("gpu join", group_rc_[g]);
		output_.set_rows(g, group_rc_[g] == PG_OK ? rows : 0);
	}
	barriers_[g]->arrive();
	if (group_rc_[g] != PG_OK) return Error;
	output_.assign(tid, g, groups_.pos_in[tid], (int) mem.size());
	return Ready;
}

Operator::GetNextResultT GpuJoinBase::getNext(unsigned short tid)
{
	if (group_rc_[groups_.group_of[tid]] != PG_OK) return std::make_pair(Error, (Page*) 0);
	return output_.next(tid);
}

Operator::ResultCode GpuJoinBase::scanStop(unsigned short tid)
{
	return DualInputOp::scanStop(tid);
}

void GpuJoinBase::threadClose(unsigned short tid)
{
	std::vector<char>().swap(build_in_[tid]);
	std::vector<char>().swap(probe_in_[tid]);
}

void GpuJoinBase::destroy()
{
	output_.clear();
	for (size_t g = 0; g < barriers_.size(); ++g) delete barriers_[g];
	barriers_.clear();
}

int GpuHashJoinOp::run_group(const pg_rel& R, const pg_rel& S, std::vector<char>& out, unsigned long long* rows)
{
	pg_ctx* ctx = shared_context();
	if (!ctx) return PG_ERR_CUDA;
	const unsigned ow = schema.getTupleSize();
	// A PK-FK join yields |S| rows: start there and grow once if asked.
	unsigned long long cap = std::max<unsigned long long>(S.n, 1);
	for (int attempt = 0; attempt < 2; ++attempt) {
		out.resize((size_t) (cap * ow));
		pg_join_result res;
		const int rc = pg_hashjoin_host(ctx, &R, &S, &cols_[0], (int) cols_.size(), &out[0], cap,
				PG_JOIN_MATERIALIZE, -1, &res);
		if (rc == PG_ERR_OUTPUT_FULL && attempt == 0) { cap = res.n_out; continue; }
		if (rc != PG_OK) return rc;
		*rows = res.n_out;
		out.resize((size_t) (res.n_out * ow));
		return PG_OK;
	}
	return PG_ERR_OUTPUT_FULL;
}

int GpuMPSMJoinOp::run_group(const pg_rel& R, const pg_rel& S, std::vector<char>& out, unsigned long long* rows)
{
	pg_ctx* ctx = shared_context();
	if (!ctx) return PG_ERR_CUDA;
	const unsigned ow = schema.getTupleSize();
	pg_stream st = 0;
	int rc = pg_stream_create(ctx, &st);
	if (rc) return rc;
	void *dR = 0, *dS = 0, *dO = 0;
	pg_join_result res;
	res.n_out = 0; res.sum = 0;
	const unsigned long long bR = R.n * R.width, bS = S.n * S.width;
	if (!(rc = pg_buffer_alloc(ctx, bR ? bR : 16, &dR)) && !(rc = pg_buffer_alloc(ctx, bS ? bS : 16, &dS)) &&
			!(rc = pg_h2d(ctx, st, dR, R.data, bR)) && !(rc = pg_h2d(ctx, st, dS, S.data, bS))) {
		pg_rel r = R, s = S;
		r.data = dR; s.data = dS;
		// Count first (exact output size), then write.
		if (!(rc = pg_mpsm_join(ctx, st, &r, &s, &cols_[0], (int) cols_.size(), 0, 0, PG_JOIN_COUNT, -1, &res))) {
			const unsigned long long n = res.n_out;
			out.resize((size_t) (n * ow));
			if (n && !(rc = pg_buffer_alloc(ctx, n * ow, &dO)) &&
					!(rc = pg_mpsm_join(ctx, st, &r, &s, &cols_[0], (int) cols_.size(), dO, n, PG_JOIN_MATERIALIZE, -1, &res)))
				rc = pg_d2h(ctx, st, &out[0], dO, n * ow);
			if (!rc) rc = pg_sync(ctx, st);
			*rows = n;
		}
	}
	if (dO) pg_buffer_free(ctx, dO);
	if (dS) pg_buffer_free(ctx, dS);
	if (dR) pg_buffer_free(ctx, dR);
	pg_stream_destroy(ctx, st);
	return rc;
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
	in_.assign(MAX_THREADS, std::vector<char>());
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

Operator::ResultCode GpuPartitionOp::scanStart(unsigned short tid, Page* idx, Schema& idxs)
{
	bool ok = nextOp->scanStart(tid, idx, idxs) != Error && drain(nextOp, tid, in_[tid]);
	if (!ok) rc_ = PG_ERR_ARG;
	barrier_.arrive();
	if (tid == 0 && rc_ == PG_OK) {
		std::vector<char> all;
		for (unsigned t = 0; t < nparts_; ++t) {
			all.insert(all.end(), in_[t].begin(), in_[t].end());
			std::vector<char>().swap(in_[t]);
		}
		const unsigned w = schema.getTupleSize();
		const unsigned long long n = w ? all.size() / w : 0;
		pg_ctx* ctx = shared_context();
		int rc = ctx ? PG_OK : PG_ERR_CUDA;
		pg_stream st = 0;
		void *din = 0, *dout = 0, *doffs = 0;
		offsets_.assign(nparts_ + 1, 0);
		if (!rc) rc = pg_stream_create(ctx, &st);
		if (!rc) rc = pg_buffer_alloc(ctx, n ? n * w : 16, &din);
		if (!rc) rc = pg_buffer_alloc(ctx, n ? n * w : 16, &dout);
		if (!rc) rc = pg_buffer_alloc(ctx, (nparts_ + 1) * 8, &doffs);
		if (!rc && n) rc = pg_h2d(ctx, st, din, &all[0], n * w);
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
			rc = pg_partition_sort(ctx, st, &p, &offsets_[0], nparts_, din);
		}
		for (unsigned t = 0; t < nparts_ && !rc; ++t) {
			std::vector<char>& o = served_.buffer((int) t);
			const unsigned long long rows = offsets_[t + 1] - offsets_[t];
			o.resize((size_t) (rows * w));
			if (rows) rc = pg_d2h(ctx, st, &o[0], (char*) dout + offsets_[t] * w, rows * w);
			served_.set_rows((int) t, rows);
		}
		if (!rc) rc = pg_sync(ctx, st);
		if (doffs) pg_buffer_free(ctx, doffs);
		if (dout) pg_buffer_free(ctx, dout);
		if (din) pg_buffer_free(ctx, din);
		if (st) pg_stream_destroy(ctx, st);
		if (rc) note_failure("gpupartition", rc);
		rc_ = rc;
	}
	barrier_.arrive();
	if (rc_ != PG_OK) return Error;
	served_.assign(tid, (int) tid, 0, 1);
	return Ready;
}

Operator::GetNextResultT GpuPartitionOp::getNext(unsigned short tid)
{
	if (rc_ != PG_OK) return std::make_pair(Error, (Page*) 0);
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
	in_.assign(MAX_THREADS, std::vector<char>());
	rc_ = PG_OK;
	output_.setup(groups_, schema.getTupleSize(), buffsize);
}

void GpuAggregateOp::threadInit(unsigned short tid)
{
	if (global_ && tid >= threads_) throw std::invalid_argument("thread id beyond `threads'");
}

int GpuAggregateOp::aggregate(const std::vector<char>& in, std::vector<char>& out, unsigned long long* groups)
{
	pg_ctx* ctx = shared_context();
	if (!ctx) return PG_ERR_CUDA;
	Schema& is = nextOp->getOutSchema();
	const unsigned w = is.getTupleSize(), ow = schema.getTupleSize();
	const unsigned long long n = w ? in.size() / w : 0;
	pg_stream st = 0;
	int rc = pg_stream_create(ctx, &st);
	if (rc) return rc;
	void *din = 0, *dout = 0;
	const unsigned long long cap = std::max<unsigned long long>(n, 1);
	uint64_t ng = 0;
	if (!(rc = pg_buffer_alloc(ctx, n ? n * w : 16, &din)) && !(rc = pg_buffer_alloc(ctx, cap * ow, &dout)) &&
			!(n && (rc = pg_h2d(ctx, st, din, &in[0], n * w)))) {
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
		if (!(rc = pg_groupby(ctx, st, &r, voff, vt, agg_, 0, dout, cap, &ng))) {
			out.resize((size_t) (ng * ow));
			if (ng) rc = pg_d2h(ctx, st, &out[0], dout, ng * ow);
			if (!rc) rc = pg_sync(ctx, st);
		}
	}
	if (dout) pg_buffer_free(ctx, dout);
	if (din) pg_buffer_free(ctx, din);
	pg_stream_destroy(ctx, st);
	*groups = ng;
	return rc;
}

Operator::ResultCode GpuAggregateOp::scanStart(unsigned short tid, Page* idx, Schema& idxs)
{
	bool ok = nextOp->scanStart(tid, idx, idxs) != Error && drain(nextOp, tid, in_[tid]);
	// The scan of the input ends inside scanStart, as GenericAggregate's does.
	if (nextOp->scanStop(tid) == Error) ok = false;
	if (!global_) {
		unsigned long long ng = 0;
		int rc = ok ? aggregate(in_[tid], output_.buffer(tid), &ng) : PG_ERR_ARG;
		std::vector<char>().swap(in_[tid]);
		if (rc) { note_failure("gpuaggregate", rc); return Error; }
		output_.set_rows(tid, ng);
		output_.assign(tid, tid, 0, 1);
		return Ready;
	}
	if (!ok) rc_ = PG_ERR_ARG;
	barrier_.arrive();
	if (tid == 0 && rc_ == PG_OK) {
		std::vector<char> all;
		for (unsigned t = 0; t < threads_; ++t) {
			all.insert(all.end(), in_[t].begin(), in_[t].end());
			std::vector<char>().swap(in_[t]);
		}
		unsigned long long ng = 0;
		rc_ = aggregate(all, output_.buffer(0), &ng);
		if (rc_) note_failure("gpuaggregate", rc_);
		output_.set_rows(0, rc_ ? 0 : ng);
	}
	barrier_.arrive();
	if (rc_ != PG_OK) return Error;
	output_.assign(tid, 0, (int) tid, (int) threads_);
	return Ready;
}

Operator::GetNextResultT GpuAggregateOp::getNext(unsigned short tid)
{
	if (global_ && rc_ != PG_OK) return std::make_pair(Error, (Page*) 0);
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

Operator* create(const std::string& type)
{
	if (type == "gpuhashjoin") return new GpuHashJoinOp();
	if (type == "gpumpsmjoin") return new GpuMPSMJoinOp();
	if (type == "gpupartition") return new GpuPartitionOp();
	if (type == "gpuaggregate_sum") return new GpuAggregateSumOp();
	if (type == "gpuaggregate_count") return new GpuAggregateCountOp();
	return 0;
}

}  // namespace pythia_gpu_ops
