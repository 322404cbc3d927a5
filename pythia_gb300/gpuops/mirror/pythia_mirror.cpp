// Mirror of the Pythia engine's Schema / Operator::init and of the libconfig++
// Setting API used by the GPU operators (see pythia_mirror.h).
#include "pythia_mirror.h"

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <time.h>
#include <sstream>

namespace libconfig {

Setting::~Setting()
{
	for (size_t i = 0; i < children_.size(); ++i) delete children_[i];
}

Setting* Setting::find(const char* name) const
{
	if (!isGroup() || !name) return 0;
	for (size_t i = 0; i < children_.size(); ++i)
		if (children_[i]->name_ == name) return children_[i];
	return 0;
}

Setting& Setting::operator[](int i) const
{
	if (!isAggregate() || i < 0 || i >= (int) children_.size())
		throw SettingNotFoundException("setting index out of range");
	return *children_[i];
}

Setting& Setting::operator[](const char* name) const
{
	Setting* s = find(name);
	if (!s) throw SettingNotFoundException(std::string("setting not found: ") + (name ? name : ""));
	return *s;
}

Setting& Setting::add(const std::string& name, Type t)
{
	if (!isAggregate()) throw SettingTypeException("add to a scalar setting");
	if (isGroup() && (name.empty() || find(name.c_str())))
		throw SettingTypeException("group members need a new, non-empty name");
	Setting* s = new Setting();
	s->type_ = t;
	s->name_ = name;
	s->parent_ = this;
	children_.push_back(s);
	return *s;
}

long long Setting::asInt() const
{
	switch (type_) {
	case TypeInt: case TypeInt64: case TypeBoolean: return ival_;
	case TypeFloat: return (long long) fval_;
	default: throw SettingTypeException("setting is not a number");
	}
}

Setting::operator bool() const
{
	if (type_ != TypeBoolean && type_ != TypeInt && type_ != TypeInt64) throw SettingTypeException("not a boolean");
	return ival_ != 0;
}
Setting::operator int() const { return (int) asInt(); }
Setting::operator unsigned int() const { return (unsigned int) asInt(); }
Setting::operator long() const { return (long) asInt(); }
Setting::operator unsigned long() const { return (unsigned long) asInt(); }
Setting::operator double() const
{
	if (type_ == TypeFloat) return fval_;
	return (double) asInt();
}
Setting::operator float() const { return (float) (double) *this; }
Setting::operator std::string() const
{
	if (type_ != TypeString) throw SettingTypeException("setting is not a string");
	return sval_;
}
Setting::operator const char*() const
{
	if (type_ != TypeString) throw SettingTypeException("setting is not a string");
	return sval_.c_str();
}

#define PG_LOOKUP(T, CONV)                                                \
	bool Setting::lookupValue(const char* name, T& v) const               \
	{                                                                     \
		Setting* s = find(name);                                          \
		if (!s) return false;                                             \
		try { v = CONV; } catch (const SettingTypeException&) { return false; } \
		return true;                                                      \
	}
PG_LOOKUP(bool, (bool) *s)
PG_LOOKUP(int, (int) *s)
PG_LOOKUP(unsigned int, (unsigned int) *s)
PG_LOOKUP(long, (long) *s)
PG_LOOKUP(unsigned long, (unsigned long) *s)
PG_LOOKUP(double, (double) *s)
PG_LOOKUP(float, (float) *s)
PG_LOOKUP(std::string, s->operator std::string())
#undef PG_LOOKUP

// ---------------------------------------------------------------------------
// libconfig text parser (recursive descent).
// ---------------------------------------------------------------------------
namespace {

struct Parser {
	const std::string& t;
	size_t i;
	int line;
	explicit Parser(const std::string& text) : t(text), i(0), line(1) { }

	void fail(const std::string& what) { throw ParseException(what, line); }

	void skip()
	{
		for (;;) {
			while (i < t.size() && isspace((unsigned char) t[i])) { if (t[i] == '\n') ++line; ++i; }
			if (i < t.size() && t[i] == '#') { while (i < t.size() && t[i] != '\n') ++i; continue; }
			if (i + 1 < t.size() && t[i] == '/' && t[i + 1] == '/') { while (i < t.size() && t[i] != '\n') ++i; continue; }
			if (i + 1 < t.size() && t[i] == '/' && t[i + 1] == '*') {
				size_t e = t.find("*/", i + 2);
				if (e == std::string::npos) fail("unterminated comment");
				for (size_t k = i; k < e; ++k) if (t[k] == '\n') ++line;
				i = e + 2;
				continue;
			}
			return;
		}
	}

	bool at(char c) { skip(); return i < t.size() && t[i] == c; }
	void expect(char c)
	{
		if (!at(c)) fail(std::string("expected '") + c + "'");
		++i;
	}

	std::string name()
	{
		skip();
		size_t b = i;
		if (i < t.size() && (isalpha((unsigned char) t[i]) || t[i] == '*')) ++i;
		else fail("expected a setting name");
		while (i < t.size() && (isalnum((unsigned char) t[i]) || t[i] == '_' || t[i] == '-' || t[i] == '*')) ++i;
		return t.substr(b, i - b);
	}

	// Members of a group until `close` (0: end of text).
	void members(Setting& g, char close)
	{
		for (;;) {
			skip();
			if (close == 0 ? i >= t.size() : at(close)) return;
			std::string n = name();
			skip();
			if (at('=') || at(':')) ++i;
			else fail("expected '=' or ':' after " + n);
			value(g, n);
			skip();
			if (at(';') || at(',')) ++i;
		}
	}

	// Elements of an array / list until `close`.
	void elements(Setting& a, char close)
	{
		for (;;) {
			if (at(close)) return;
			value(a, std::string());
			if (at(',')) { ++i; continue; }
			if (!at(close)) fail(std::string("expected ',' or '") + close + "'");
		}
	}

	void value(Setting& parent, const std::string& n)
	{
		skip();
		if (i >= t.size()) fail("expected a value");
		const char c = t[i];
		if (c == '{') { ++i; Setting& g = parent.add(n, Setting::TypeGroup); members(g, '}'); expect('}'); return; }
		if (c == '[') { ++i; Setting& a = parent.add(n, Setting::TypeArray); elements(a, ']'); expect(']'); return; }
		if (c == '(') { ++i; Setting& l = parent.add(n, Setting::TypeList); elements(l, ')'); expect(')'); return; }
		if (c == '"') {
			std::string s;
			while (at('"')) {
				++i;
				while (i < t.size() && t[i] != '"') {
					if (t[i] == '\\' && i + 1 < t.size()) {
						++i;
						const char e = t[i];
						s += e == 'n' ? '\n' : e == 't' ? '\t' : e;
					} else {
						s += t[i];
					}
					++i;
				}
				if (i >= t.size()) fail("unterminated string");
				++i;
			}
			parent.add(n, Setting::TypeString) = s;
			return;
		}
		size_t b = i;
		while (i < t.size() && (isalnum((unsigned char) t[i]) || t[i] == '.' || t[i] == '-' || t[i] == '+')) ++i;
		std::string w = t.substr(b, i - b);
		std::string lw = w;
		std::transform(lw.begin(), lw.end(), lw.begin(), ::tolower);
		if (lw == "true" || lw == "false") { parent.add(n, Setting::TypeBoolean) = (lw == "true"); return; }
		if (w.empty()) fail("expected a value");
		const bool hex = lw.size() > 2 && lw[0] == '0' && lw[1] == 'x';
		const bool isfloat = !hex && (lw.find('.') != std::string::npos || lw.find('e') != std::string::npos);
		if (isfloat) {
			char* end = 0;
			const double d = strtod(w.c_str(), &end);
			if (*end) fail("bad number " + w);
			parent.add(n, Setting::TypeFloat) = d;
			return;
		}
		bool is64 = false;
		if (!lw.empty() && lw[lw.size() - 1] == 'l') { is64 = true; w.erase(w.size() - 1); }
		char* end = 0;
		const long long v = strtoll(w.c_str(), &end, hex ? 16 : 10);
		if (*end) fail("bad number " + w);
		if (is64 || v > 2147483647LL || v < -2147483647LL - 1) parent.add(n, Setting::TypeInt64) = (long) v;
		else parent.add(n, Setting::TypeInt) = (int) v;
	}
};

}  // namespace

void Config::readString(const std::string& text)
{
	Parser p(text);
	p.members(root_, 0);
}

Setting& Config::lookup(const std::string& path) const
{
	Setting* s = &getRoot();
	size_t b = 0;
	while (b <= path.size()) {
		size_t e = path.find('.', b);
		if (e == std::string::npos) e = path.size();
		s = &(*s)[path.substr(b, e - b)];
		b = e + 1;
	}
	return *s;
}

bool Config::exists(const std::string& path) const
{
	try { lookup(path); return true; } catch (const SettingNotFoundException&) { return false; }
}

}  // namespace libconfig

// ---------------------------------------------------------------------------
// Schema and Operator::init.
// ---------------------------------------------------------------------------
void Schema::add(ColumnType ct, unsigned int size)
{
	unsigned int w = 0;
	switch (ct) {
	case CT_INTEGER: w = sizeof(CtInt); break;
	case CT_LONG: w = sizeof(CtLong); break;
	case CT_DECIMAL: w = sizeof(CtDecimal); break;
	case CT_DATE: w = sizeof(CtLong); break;
	case CT_POINTER: w = sizeof(void*); break;
	case CT_CHAR: w = size; break;
	}
	vct.push_back(ct);
	voffset.push_back(totalsize);
	vformat.push_back(std::string());
	totalsize += w;
}

void Schema::add(ColumnType ct, const std::string& formatstr)
{
	add(ct, 0);
	vformat.back() = formatstr;
}

void Schema::add(ColumnSpec desc)
{
	if (desc.type == CT_DATE) add(CT_DATE, desc.formatstr);
	else add(desc.type, desc.size);
}

void Schema::parseTuple(void* dest, const char** input) const
{
	for (unsigned int i = 0; i < columns(); ++i) {
		char* d = (char*) dest + voffset[i];
		switch (vct[i]) {
		case CT_INTEGER: { int v = atoi(input[i]); memcpy(d, &v, sizeof v); break; }
		case CT_LONG: { long long v = atoll(input[i]); memcpy(d, &v, sizeof v); break; }
		case CT_DECIMAL: { double v = atof(input[i]); memcpy(d, &v, sizeof v); break; }
		case CT_CHAR: strncpy(d, input[i], getColumnWidth(i)); break;
		case CT_DATE: {
			// Packed fields, least significant first: 20 bits below the
			// seconds, then seconds and minutes (6 bits), hours and days (5),
			// months (4) and years since 1900 (18).
			struct tm t;
			memset(&t, 0, sizeof t);
			strptime(input[i], vformat[i].c_str(), &t);
			unsigned long long v = 0;
			v |= ((unsigned long long) t.tm_sec & 0x3Full) << 20;
			v |= ((unsigned long long) t.tm_min & 0x3Full) << 26;
			v |= ((unsigned long long) t.tm_hour & 0x1Full) << 32;
			v |= ((unsigned long long) t.tm_mday & 0x1Full) << 37;
			v |= ((unsigned long long) t.tm_mon & 0xFull) << 42;
			v |= ((unsigned long long) t.tm_year & 0x3FFFFull) << 46;
			memcpy(d, &v, sizeof v);
			break;
		}
		case CT_POINTER: throw std::invalid_argument("pointer columns have no text form");
		}
	}
}

Schema Schema::create(const libconfig::Setting& line)
{
	Schema ret;
	for (int k = 0; k < line.getLength(); ++k) {
		std::string v = line[k];
		std::string::size_type paren = v.find('(');
		std::string head = v.substr(0, paren);
		std::transform(head.begin(), head.end(), head.begin(), ::tolower);
		if (head.find("int") == 0) ret.add(CT_INTEGER);
		else if (head.find("long") == 0) ret.add(CT_LONG);
		else if (head.find("dec") == 0) ret.add(CT_DECIMAL);
		else if (head.find("date") == 0) {
			if (paren == std::string::npos) throw std::invalid_argument("date needs a format: " + v);
			ret.add(CT_DATE, v.substr(paren + 1));
		} else if (head.find("char") == 0) {
			if (paren == std::string::npos) throw std::invalid_argument("char needs a length: " + v);
			std::istringstream is(v.substr(paren + 1));
			int len = 0;
			is >> len;
			if (!is || len < 0) throw std::invalid_argument("bad char length: " + v);
			ret.add(CT_CHAR, (unsigned int) len + 1);   // room for the terminating zero
		} else {
			throw std::invalid_argument("unknown column type: " + v);
		}
	}
	return ret;
}

void Operator::init(libconfig::Config& root, libconfig::Setting& node)
{
	(void) node;
	buffsize = root.getRoot()["buffsize"];
}
