// Host-side mirror of the Pythia operator interface, for builds without the
// Pythia source tree (the GPU host). It declares the same names with the same
// meaning as the reference engine: Operator with its ResultCode / Page /
// GetNextResultT types and init / threadInit / scanStart / getNext / scanStop /
// threadClose / destroy virtuals (operators/operators.h:79-186),
// SingleInputOp::nextOp, DualInputOp::buildOp / probeOp, ZeroInputOp;
// TupleBuffer pages (util/buffer.h:134-337: data, free, maxsize, tuplesize,
// getTupleOffset returning 0 past the used space); Schema with the packed
// row layout and type sizes of schema.h:161-350 (int 4, long 8, dec 8,
// char(n) n+1, date 8, pointer 8) and Schema::create from a list of type
// strings (schema.cpp:221-260); and the part of libconfig++'s Setting / Config
// API the GPU operators read (lookup by name and index, getLength, exists,
// lookupValue, scalar conversions), with a parser for the libconfig text
// format the plans are written in. Written in C++98 like the engine.
#ifndef PYTHIA_MIRROR_H
#define PYTHIA_MIRROR_H

#include <map>
#include <string>
#include <utility>
#include <vector>
#include <stdexcept>
#include <cstring>
#include <stdint.h>

namespace libconfig {

class SettingNotFoundException : public std::runtime_error {
public:
	explicit SettingNotFoundException(const std::string& what) : std::runtime_error(what) { }
};

class SettingTypeException : public std::runtime_error {
public:
	explicit SettingTypeException(const std::string& what) : std::runtime_error(what) { }
};

class ParseException : public std::runtime_error {
public:
	ParseException(const std::string& what, int line) : std::runtime_error(what), line_(line) { }
	int getLine() const { return line_; }
private:
	int line_;
};

class Setting {
public:
	enum Type { TypeNone, TypeInt, TypeInt64, TypeFloat, TypeString, TypeBoolean, TypeGroup, TypeArray, TypeList };

	Setting() : type_(TypeGroup), ival_(0), fval_(0.0), parent_(0) { }
	~Setting();

	Type getType() const { return type_; }
	bool isGroup() const { return type_ == TypeGroup; }
	bool isArray() const { return type_ == TypeArray; }
	bool isList() const { return type_ == TypeList; }
	bool isAggregate() const { return isGroup() || isArray() || isList(); }
	bool isNumber() const { return type_ == TypeInt || type_ == TypeInt64 || type_ == TypeFloat; }
	bool isScalar() const { return !isAggregate() && type_ != TypeNone; }
	int getLength() const { return isAggregate() ? (int) children_.size() : 0; }
	const char* getName() const { return name_.empty() ? 0 : name_.c_str(); }

	Setting& operator[](int i) const;
	Setting& operator[](const char* name) const;
	Setting& operator[](const std::string& name) const { return (*this)[name.c_str()]; }
	bool exists(const char* name) const { return find(name) != 0; }
	bool exists(const std::string& name) const { return exists(name.c_str()); }

	bool lookupValue(const char* name, bool& v) const;
	bool lookupValue(const char* name, int& v) const;
	bool lookupValue(const char* name, unsigned int& v) const;
	bool lookupValue(const char* name, long& v) const;
	bool lookupValue(const char* name, unsigned long& v) const;
	bool lookupValue(const char* name, double& v) const;
	bool lookupValue(const char* name, float& v) const;
	bool lookupValue(const char* name, std::string& v) const;

	operator bool() const;
	operator int() const;
	operator unsigned int() const;
	operator long() const;
	operator unsigned long() const;
	operator double() const;
	operator float() const;
	operator std::string() const;
	operator const char*() const;

	// Building (used by the parser and by programs that make plans in code).
	Setting& add(const std::string& name, Type t);
	Setting& add(Type t) { return add(std::string(), t); }
	Setting& operator=(long v) { type_ = TypeInt64; ival_ = v; fval_ = (double) v; return *this; }
	Setting& operator=(int v) { type_ = TypeInt; ival_ = v; fval_ = v; return *this; }
	Setting& operator=(const double& v) { type_ = TypeFloat; fval_ = v; ival_ = (long long) v; return *this; }
	Setting& operator=(float v) { return (*this) = (double) v; }
	Setting& operator=(bool v) { type_ = TypeBoolean; ival_ = v; return *this; }
	Setting& operator=(const std::string& v) { type_ = TypeString; sval_ = v; return *this; }
	Setting& operator=(const char* v) { return (*this) = std::string(v); }

private:
	Setting(const Setting&);
	Setting& operator=(const Setting&);
	Setting* find(const char* name) const;
	long long asInt() const;

	Type type_;
	std::string name_;
	long long ival_;
	double fval_;
	std::string sval_;
	std::vector<Setting*> children_;
	Setting* parent_;
};

class Config {
public:
	Config() { }
	Setting& getRoot() const { return const_cast<Setting&>(root_); }
	// Parses libconfig text: `name = value;` (or `:`), groups { }, arrays [ ],
	// lists ( ), strings (adjacent ones concatenate), integers (decimal or 0x,
	// optional L), floats, true/false, and # // /* */ comments.
	void readString(const std::string& text);
	void readString(const char* text) { readString(std::string(text)); }
	// Dotted path lookup, e.g. "join.build" (names only).
	Setting& lookup(const std::string& path) const;
	bool exists(const std::string& path) const;
private:
	Config(const Config&);
	Config& operator=(const Config&);
	Setting root_;
};

}  // namespace libconfig

enum ColumnType {
	CT_INTEGER,
	CT_LONG,
	CT_DECIMAL,
	CT_CHAR,
	CT_DATE,
	CT_POINTER
};

typedef int CtInt;
typedef long long CtLong;
typedef double CtDecimal;
typedef char CtChar;

// A column: type, width, and (dates) the strptime format of its text form.
struct ColumnSpec {
	ColumnSpec(ColumnType ct, unsigned int sz, const std::string& str = std::string())
		: type(ct), size(sz), formatstr(str) { }
	ColumnType type;
	unsigned int size;
	std::string formatstr;
};

class Schema {
public:
	Schema() : totalsize(0) { }
	void add(ColumnType ct, unsigned int size = 0);
	void add(ColumnType ct, const std::string& formatstr);
	void add(ColumnSpec desc);
	ColumnType getColumnType(unsigned int pos) const { return vct.at(pos); }
	ColumnSpec get(unsigned int pos) const { return ColumnSpec(vct.at(pos), getColumnWidth(pos), vformat.at(pos)); }
	// Text to tuple, one string per column: int/long/dec as atoi/atoll/atof,
	// char copied with strncpy into the column, date through strptime and the
	// engine's packed date form (schema.cpp:129-168, schema.h:66-104).
	void parseTuple(void* dest, const char** input) const;
	unsigned int getColumnWidth(unsigned int pos) const
	{
		return (pos + 1 < voffset.size() ? voffset[pos + 1] : totalsize) - voffset.at(pos);
	}
	unsigned int columns() const { return (unsigned int) vct.size(); }
	unsigned int getTupleSize() const { return totalsize; }
	void* calcOffset(void* data, unsigned int pos) const { return (char*) data + voffset.at(pos); }
	void copyTuple(void* dest, const void* src) const { memcpy(dest, src, totalsize); }
	static Schema create(const libconfig::Setting& line);
private:
	std::vector<ColumnType> vct;
	std::vector<unsigned int> voffset;
	std::vector<std::string> vformat;
	unsigned int totalsize;
};

// A page: `maxsize` bytes at `data`, the bytes before `free` hold tuples of
// `tuplesize` bytes. Pages made from a pointer do not own their memory.
class TupleBuffer {
public:
	TupleBuffer(void* data, unsigned long long size, void* free, unsigned int tuplesize)
		: data_((char*) data), maxsize_(size), free_((char*) (free ? free : data)), tuplesize_(tuplesize), owner_(false) { }
	TupleBuffer(unsigned long long size, unsigned int tuplesize, void* allocsource = 0, const char tag[4] = "Buff")
		: data_(new char[size ? size : 1]), maxsize_(size), free_(0), tuplesize_(tuplesize), owner_(true)
	{
		(void) allocsource; (void) tag;
		free_ = data_;
	}
	~TupleBuffer() { if (owner_) delete[] data_; }

	bool canStore(unsigned long long len) const { return free_ + len <= data_ + maxsize_; }
	bool canStoreTuple() const { return canStore(tuplesize_); }
	void* allocate(unsigned long long len)
	{
		if (!canStore(len)) return 0;
		void* r = free_;
		free_ += len;
		return r;
	}
	void* allocateTuple() { return allocate(tuplesize_); }
	void clear() { free_ = data_; }
	unsigned long long capacity() const { return maxsize_; }
	unsigned long long getUsedSpace() const { return (unsigned long long) (free_ - data_); }
	void* getTupleOffset(unsigned long long pos) const
	{
		char* p = data_ + pos * tuplesize_;
		return p < free_ ? p : 0;
	}
	bool isValidTupleAddress(void* loc) const { return (char*) loc >= data_ && (char*) loc + tuplesize_ <= free_; }
	unsigned int getTupleSize() const { return tuplesize_; }
private:
	TupleBuffer(const TupleBuffer&);
	TupleBuffer& operator=(const TupleBuffer&);
	char* data_;
	unsigned long long maxsize_;
	char* free_;
	unsigned int tuplesize_;
	bool owner_;
};

class SingleInputOp;
class DualInputOp;
class ZeroInputOp;

class Visitor {
public:
	virtual ~Visitor() { }
	virtual void visit(SingleInputOp* op) { (void) op; }
	virtual void visit(DualInputOp* op) { (void) op; }
	virtual void visit(ZeroInputOp* op) { (void) op; }
};

static const unsigned short MAX_THREADS = 128;

class Operator {
public:
	Operator() : buffsize(0) { }
	enum ResultCode { Ready = 0, Finished, Error };
	typedef TupleBuffer Page;
	typedef std::pair<Operator::ResultCode, Page*> GetNextResultT;

	virtual ~Operator() { }
	virtual void init(libconfig::Config& root, libconfig::Setting& node);
	virtual void threadInit(unsigned short threadid) { (void) threadid; }
	virtual ResultCode scanStart(unsigned short threadid, Page* indexdatapage, Schema& indexdataschema) = 0;
	virtual GetNextResultT getNext(unsigned short threadid) = 0;
	virtual ResultCode scanStop(unsigned short threadid) = 0;
	virtual void threadClose(unsigned short threadid) { (void) threadid; }
	virtual void destroy() { }
	virtual void accept(Visitor* v) = 0;
	virtual Schema& getOutSchema() { return schema; }
protected:
	Schema schema;
	unsigned int buffsize;
};

class SingleInputOp : public virtual Operator {
public:
	SingleInputOp() : nextOp(0) { }
	virtual ~SingleInputOp() { }
	virtual void accept(Visitor* v) { v->visit(this); }
	virtual ResultCode scanStart(unsigned short threadid, Page* indexdatapage, Schema& indexdataschema)
	{
		return nextOp->scanStart(threadid, indexdatapage, indexdataschema);
	}
	virtual ResultCode scanStop(unsigned short threadid) { return nextOp->scanStop(threadid); }
	Operator* nextOp;
};

class DualInputOp : public virtual Operator {
public:
	DualInputOp() : buildOp(0), probeOp(0) { }
	virtual ~DualInputOp() { }
	virtual void accept(Visitor* v) { v->visit(this); }
	virtual ResultCode scanStart(unsigned short threadid, Page* indexdatapage, Schema& indexdataschema)
	{
		ResultCode a = buildOp->scanStart(threadid, indexdatapage, indexdataschema);
		ResultCode b = probeOp->scanStart(threadid, indexdatapage, indexdataschema);
		return a == b ? a : Operator::Error;
	}
	virtual ResultCode scanStop(unsigned short threadid)
	{
		ResultCode a = buildOp->scanStop(threadid);
		ResultCode b = probeOp->scanStop(threadid);
		return a == b ? a : Operator::Error;
	}
	Operator* buildOp;
	Operator* probeOp;
};

class ZeroInputOp : public virtual Operator {
public:
	virtual ~ZeroInputOp() { }
	virtual void accept(Visitor* v) { v->visit(this); }
	virtual ResultCode scanStart(unsigned short threadid, Page* indexdatapage, Schema& indexdataschema)
	{
		(void) threadid; (void) indexdatapage; (void) indexdataschema;
		return Ready;
	}
	virtual ResultCode scanStop(unsigned short threadid) { (void) threadid; return Ready; }
};

#endif
