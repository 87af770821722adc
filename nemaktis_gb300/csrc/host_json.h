// Minimal JSON reader for the bpm backend settings string.
//
// The reference parses its settings with a vendored nlohmann::json
// (BeamPropagationSolver/src/UtilitiesLib/json.h, third-party); this is an independent,
// small recursive-descent reader for RFC 8259 documents: objects, arrays, strings (with
// escapes), numbers, true/false/null. Errors throw nbpm::JsonError with a byte offset.
#pragma once

#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace nbpm {

struct JsonError : std::runtime_error {
	using std::runtime_error::runtime_error;
};

struct Json {
	enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
	bool b = false;
	double num = 0;
	bool is_int = false;
	std::string str;
	std::vector<Json> arr;
	std::vector<std::pair<std::string, Json>> obj;  // insertion order

	bool has(const std::string& k) const {
		for(auto& kv : obj) if(kv.first == k) return true;
		return false;
	}
	const Json& at(const std::string& k) const {
		if(kind != Object) throw JsonError("type_error: cannot use at() with a non-object value");
		for(auto& kv : obj) if(kv.first == k) return kv.second;
		throw JsonError("out_of_range: key '" + k + "' not found");
	}
	const char* kind_name() const {
		static const char* n[] = {"null", "boolean", "number", "string", "array", "object"};
		return n[kind];
	}
	double as_number() const {
		if(kind != Number) throw JsonError(std::string("type_error: type must be number, but is ") + kind_name());
		return num;
	}
	long long as_int() const { return (long long)as_number(); }
	bool as_bool() const {
		if(kind != Bool) throw JsonError(std::string("type_error: type must be boolean, but is ") + kind_name());
		return b;
	}
	const std::string& as_string() const {
		if(kind != String) throw JsonError(std::string("type_error: type must be string, but is ") + kind_name());
		return str;
	}
	std::vector<double> as_number_array() const {
		if(kind != Array) throw JsonError(std::string("type_error: type must be array, but is ") + kind_name());
		std::vector<double> v;
		for(auto& e : arr) v.push_back(e.as_number());
		return v;
	}
};

class JsonReader {
public:
	static Json parse(const std::string& s) {
		JsonReader r(s);
		r.ws();
		Json v = r.value(0);
		r.ws();
		if(r.i != s.size()) r.fail("unexpected trailing characters");
		return v;
	}

private:
	explicit JsonReader(const std::string& s) : s(s), i(0) {}
	const std::string& s;
	size_t i;

	[[noreturn]] void fail(const std::string& what) {
		throw JsonError("parse_error: " + what + " at byte " + std::to_string(i));
	}
	void ws() {
		while(i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\r')) i++;
	}
	bool lit(const char* w) {
		size_t n = std::char_traits<char>::length(w);
		if(s.compare(i, n, w) == 0) { i += n; return true; }
		return false;
	}
	Json value(int depth) {
		if(depth > 256) fail("nesting too deep");
		if(i >= s.size()) fail("unexpected end of input");
		char c = s[i];
		Json v;
		if(c == '{') {
			v.kind = Json::Object;
			i++; ws();
			if(i < s.size() && s[i] == '}') { i++; return v; }
			while(true) {
				ws();
				if(i >= s.size() || s[i] != '"') fail("expected string key");
				std::string k = string_lit();
				ws();
				if(i >= s.size() || s[i] != ':') fail("expected ':'");
				i++; ws();
				Json e = value(depth + 1);
				bool replaced = false;
				for(auto& kv : v.obj) if(kv.first == k) { kv.second = e; replaced = true; }
				if(!replaced) v.obj.emplace_back(k, std::move(e));
				ws();
				if(i < s.size() && s[i] == ',') { i++; continue; }
				if(i < s.size() && s[i] == '}') { i++; return v; }
				fail("expected ',' or '}'");
			}
		}
		if(c == '[') {
			v.kind = Json::Array;
			i++; ws();
			if(i < s.size() && s[i] == ']') { i++; return v; }
			while(true) {
				ws();
				v.arr.push_back(value(depth + 1));
				ws();
				if(i < s.size() && s[i] == ',') { i++; continue; }
				if(i < s.size() && s[i] == ']') { i++; return v; }
				fail("expected ',' or ']'");
			}
		}
		if(c == '"') { v.kind = Json::String; v.str = string_lit(); return v; }
		if(lit("true")) { v.kind = Json::Bool; v.b = true; return v; }
		if(lit("false")) { v.kind = Json::Bool; v.b = false; return v; }
		if(lit("null")) { v.kind = Json::Null; return v; }
		if(c == '-' || (c >= '0' && c <= '9')) {
			size_t st = i;
			if(s[i] == '-') i++;
			if(i >= s.size() || !(s[i] >= '0' && s[i] <= '9')) fail("invalid number");
			bool integral = true;
			while(i < s.size() && s[i] >= '0' && s[i] <= '9') i++;
			if(i < s.size() && s[i] == '.') {
				integral = false; i++;
				if(i >= s.size() || !(s[i] >= '0' && s[i] <= '9')) fail("invalid number");
				while(i < s.size() && s[i] >= '0' && s[i] <= '9') i++;
			}
			if(i < s.size() && (s[i] == 'e' || s[i] == 'E')) {
				integral = false; i++;
				if(i < s.size() && (s[i] == '+' || s[i] == '-')) i++;
				if(i >= s.size() || !(s[i] >= '0' && s[i] <= '9')) fail("invalid number");
				while(i < s.size() && s[i] >= '0' && s[i] <= '9') i++;
			}
			v.kind = Json::Number;
			v.is_int = integral;
			v.num = std::strtod(s.substr(st, i - st).c_str(), nullptr);
			return v;
		}
		fail("unexpected character");
	}
	static void utf8(std::string& out, unsigned cp) {
		if(cp < 0x80) out += (char)cp;
		else if(cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
		else if(cp < 0x10000) {
			out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F));
			out += (char)(0x80 | (cp & 0x3F));
		}
		else {
			out += (char)(0xF0 | (cp >> 18)); out += (char)(0x80 | ((cp >> 12) & 0x3F));
			out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F));
		}
	}
	unsigned hex4() {
		if(i + 4 > s.size()) fail("bad unicode escape");
		unsigned v = 0;
		for(int k = 0; k < 4; k++) {
			char c = s[i++];
			v <<= 4;
			if(c >= '0' && c <= '9') v |= c - '0';
			else if(c >= 'a' && c <= 'f') v |= c - 'a' + 10;
			else if(c >= 'A' && c <= 'F') v |= c - 'A' + 10;
			else fail("bad unicode escape");
		}
		return v;
	}
	std::string string_lit() {
		std::string out;
		i++;  // opening quote
		while(true) {
			if(i >= s.size()) fail("unterminated string");
			char c = s[i++];
			if(c == '"') return out;
			if((unsigned char)c < 0x20) fail("control character in string");
			if(c != '\\') { out += c; continue; }
			if(i >= s.size()) fail("unterminated escape");
			char e = s[i++];
			switch(e) {
				case '"': out += '"'; break;
				case '\\': out += '\\'; break;
				case '/': out += '/'; break;
				case 'b': out += '\b'; break;
				case 'f': out += '\f'; break;
				case 'n': out += '\n'; break;
				case 'r': out += '\r'; break;
				case 't': out += '\t'; break;
				case 'u': {
					unsigned cp = hex4();
					if(cp >= 0xD800 && cp <= 0xDBFF) {
						if(i + 2 <= s.size() && s[i] == '\\' && s[i + 1] == 'u') {
							i += 2;
							unsigned lo = hex4();
							cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
						}
					}
					utf8(out, cp);
					break;
				}
				default: fail("bad escape");
			}
		}
	}
};

}  // namespace nbpm
