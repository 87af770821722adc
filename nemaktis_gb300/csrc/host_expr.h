// Arithmetic-expression compiler/evaluator for refractive-index and mask formulas.
//
// The reference hands these strings to muParser (PhysicsCoefficients.cpp:27-103 with the
// variable "lambda" in µm; VectorField.cpp:72-76 with "x", "y", "z"). muParser is an
// external dependency; this file implements the subset of its documented grammar that the
// Nemaktis front end emits, compiled once to a postfix program and evaluated in FP64:
//   ternary  := or ('?' ternary ':' ternary)?
//   or/and   := '||' / '&&'        cmp := '<' '>' '<=' '>=' '==' '!='
//   add      := mul (('+'|'-') mul)*      mul := unary (('*'|'/') unary)*
//   unary    := ('-'|'+') unary | power   power := primary ('^' unary)?   (right assoc.)
//   primary  := number | variable | _pi | _e | func '(' args ')' | '(' ternary ')'
// Functions: sin cos tan asin acos atan sinh cosh tanh asinh acosh atanh log2 log10 log ln
// exp sqrt sign rint abs (one argument) and min max sum avg (one or more arguments).
#pragma once

#include <cctype>
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

namespace nbpm {

struct ExprError : std::runtime_error {
	using std::runtime_error::runtime_error;
};

class Expr {
public:
	Expr() = default;
	Expr(const std::string& src, const std::vector<std::string>& vars) : vars_(vars) {
		s_ = src;
		pos_ = 0;
		next();
		ternary();
		if(tok_ != T_END) throw ExprError("unexpected token in expression \"" + src + "\"");
	}

	double eval(const double* v) const {
		double st[64];
		int sp = 0;
		for(const Op& o : prog_) {
			switch(o.code) {
				case C_NUM: st[sp++] = o.val; break;
				case C_VAR: st[sp++] = v[o.arg]; break;
				case C_NEG: st[sp - 1] = -st[sp - 1]; break;
				case C_ADD: sp--; st[sp - 1] += st[sp]; break;
				case C_SUB: sp--; st[sp - 1] -= st[sp]; break;
				case C_MUL: sp--; st[sp - 1] *= st[sp]; break;
				case C_DIV: sp--; st[sp - 1] /= st[sp]; break;
				case C_POW: sp--; st[sp - 1] = std::pow(st[sp - 1], st[sp]); break;
				case C_LT: sp--; st[sp - 1] = st[sp - 1] < st[sp]; break;
				case C_GT: sp--; st[sp - 1] = st[sp - 1] > st[sp]; break;
				case C_LE: sp--; st[sp - 1] = st[sp - 1] <= st[sp]; break;
				case C_GE: sp--; st[sp - 1] = st[sp - 1] >= st[sp]; break;
				case C_EQ: sp--; st[sp - 1] = st[sp - 1] == st[sp]; break;
				case C_NE: sp--; st[sp - 1] = st[sp - 1] != st[sp]; break;
				case C_AND: sp--; st[sp - 1] = (st[sp - 1] != 0) && (st[sp] != 0); break;
				case C_OR: sp--; st[sp - 1] = (st[sp - 1] != 0) || (st[sp] != 0); break;
				case C_SEL: sp -= 2; st[sp - 1] = (st[sp - 1] != 0) ? st[sp] : st[sp + 1]; break;
				case C_F1: st[sp - 1] = fn1(o.arg, st[sp - 1]); break;
				case C_FN: {
					int n = (int)o.val;
					sp -= n;
					double r = st[sp];
					for(int k = 1; k < n; k++) {
						double x = st[sp + k];
						if(o.arg == 0) r = std::fmin(r, x);
						else if(o.arg == 1) r = std::fmax(r, x);
						else r += x;
					}
					if(o.arg == 3) r /= n;
					st[sp++] = r;
					break;
				}
			}
		}
		return st[0];
	}
	double eval1(double a) const { return eval(&a); }

private:
	enum Code { C_NUM, C_VAR, C_NEG, C_ADD, C_SUB, C_MUL, C_DIV, C_POW, C_LT, C_GT, C_LE, C_GE,
		C_EQ, C_NE, C_AND, C_OR, C_SEL, C_F1, C_FN };
	struct Op { Code code; int arg; double val; };
	enum Tok { T_END, T_NUM, T_NAME, T_OP };

	std::vector<std::string> vars_;
	std::vector<Op> prog_;
	std::string s_;
	size_t pos_ = 0;
	Tok tok_ = T_END;
	std::string tv_;
	double tnum_ = 0;
	int depth_ = 0, maxdepth_ = 0;

	static double fn1(int id, double x) {
		switch(id) {
			case 0: return std::sin(x); case 1: return std::cos(x); case 2: return std::tan(x);
			case 3: return std::asin(x); case 4: return std::acos(x); case 5: return std::atan(x);
			case 6: return std::sinh(x); case 7: return std::cosh(x); case 8: return std::tanh(x);
			case 9: return std::asinh(x); case 10: return std::acosh(x); case 11: return std::atanh(x);
			case 12: return std::log2(x); case 13: return std::log10(x); case 14: return std::log(x);
			case 15: return std::log(x); case 16: return std::exp(x); case 17: return std::sqrt(x);
			case 18: return (x > 0) - (x < 0); case 19: return std::rint(x); case 20: return std::fabs(x);
		}
		return NAN;
	}
	static int fn1_id(const std::string& n) {
		static const char* names[] = {"sin", "cos", "tan", "asin", "acos", "atan", "sinh", "cosh",
			"tanh", "asinh", "acosh", "atanh", "log2", "log10", "log", "ln", "exp", "sqrt", "sign",
			"rint", "abs"};
		for(int k = 0; k < 21; k++) if(n == names[k]) return k;
		return -1;
	}
	void emit(Code c, int arg = 0, double val = 0) {
		prog_.push_back({c, arg, val});
		int d = 0;
		switch(c) {
			case C_NUM: case C_VAR: d = 1; break;
			case C_NEG: case C_F1: d = 0; break;
			case C_SEL: d = -2; break;
			case C_FN: d = 1 - (int)val; break;
			default: d = -1;
		}
		depth_ += d;
		if(depth_ > maxdepth_) maxdepth_ = depth_;
		if(maxdepth_ > 60) throw ExprError("expression too deep: \"" + s_ + "\"");
	}
	[[noreturn]] void fail(const std::string& w) {
		throw ExprError(w + " in expression \"" + s_ + "\"");
	}
	void next() {
		while(pos_ < s_.size() && std::isspace((unsigned char)s_[pos_])) pos_++;
		if(pos_ >= s_.size()) { tok_ = T_END; return; }
		char c = s_[pos_];
		if(std::isdigit((unsigned char)c) || (c == '.' && pos_ + 1 < s_.size() && std::isdigit((unsigned char)s_[pos_ + 1]))) {
			size_t st = pos_;
			while(pos_ < s_.size() && (std::isdigit((unsigned char)s_[pos_]) || s_[pos_] == '.')) pos_++;
			if(pos_ < s_.size() && (s_[pos_] == 'e' || s_[pos_] == 'E')) {
				size_t save = pos_;
				pos_++;
				if(pos_ < s_.size() && (s_[pos_] == '+' || s_[pos_] == '-')) pos_++;
				if(pos_ < s_.size() && std::isdigit((unsigned char)s_[pos_])) {
					while(pos_ < s_.size() && std::isdigit((unsigned char)s_[pos_])) pos_++;
				}
				else pos_ = save;
			}
			tok_ = T_NUM;
			std::string t = s_.substr(st, pos_ - st);
			char* end = nullptr;
			tnum_ = std::strtod(t.c_str(), &end);
			if(!end || *end) fail("bad number \"" + t + "\"");
			return;
		}
		if(std::isalpha((unsigned char)c) || c == '_') {
			size_t st = pos_;
			while(pos_ < s_.size() && (std::isalnum((unsigned char)s_[pos_]) || s_[pos_] == '_')) pos_++;
			tok_ = T_NAME;
			tv_ = s_.substr(st, pos_ - st);
			return;
		}
		static const char* two[] = {"||", "&&", "<=", ">=", "==", "!="};
		for(auto t : two)
			if(s_.compare(pos_, 2, t) == 0) { tok_ = T_OP; tv_ = t; pos_ += 2; return; }
		if(std::string("+-*/^(),<>?:").find(c) != std::string::npos) {
			tok_ = T_OP; tv_ = std::string(1, c); pos_++; return;
		}
		fail(std::string("unexpected character '") + c + "'");
	}
	bool is_op(const char* o) const { return tok_ == T_OP && tv_ == o; }
	void expect(const char* o) {
		if(!is_op(o)) fail(std::string("expected '") + o + "'");
		next();
	}
	void ternary() {
		lor();
		if(is_op("?")) {
			next();
			ternary();
			expect(":");
			ternary();
			emit(C_SEL);
		}
	}
	void lor() { land(); while(is_op("||")) { next(); land(); emit(C_OR); } }
	void land() { cmp(); while(is_op("&&")) { next(); cmp(); emit(C_AND); } }
	void cmp() {
		add();
		while(true) {
			Code c;
			if(is_op("<")) c = C_LT; else if(is_op(">")) c = C_GT; else if(is_op("<=")) c = C_LE;
			else if(is_op(">=")) c = C_GE; else if(is_op("==")) c = C_EQ; else if(is_op("!=")) c = C_NE;
			else return;
			next(); add(); emit(c);
		}
	}
	void add() {
		mul();
		while(is_op("+") || is_op("-")) {
			Code c = is_op("+") ? C_ADD : C_SUB;
			next(); mul(); emit(c);
		}
	}
	void mul() {
		unary();
		while(is_op("*") || is_op("/")) {
			Code c = is_op("*") ? C_MUL : C_DIV;
			next(); unary(); emit(c);
		}
	}
	void unary() {
		if(is_op("-")) { next(); unary(); emit(C_NEG); return; }
		if(is_op("+")) { next(); unary(); return; }
		power();
	}
	void power() {
		primary();
		if(is_op("^")) { next(); unary(); emit(C_POW); }
	}
	void primary() {
		if(tok_ == T_NUM) { emit(C_NUM, 0, tnum_); next(); return; }
		if(is_op("(")) { next(); ternary(); expect(")"); return; }
		if(tok_ == T_NAME) {
			std::string name = tv_;
			next();
			if(is_op("(")) {
				next();
				int nargs = 1;
				ternary();
				while(is_op(",")) { next(); ternary(); nargs++; }
				expect(")");
				int id = fn1_id(name);
				if(id >= 0) {
					if(nargs != 1) fail("function " + name + " takes one argument");
					emit(C_F1, id);
					return;
				}
				int vid = name == "min" ? 0 : name == "max" ? 1 : name == "sum" ? 2 : name == "avg" ? 3 : -1;
				if(vid < 0) fail("unknown function \"" + name + "\"");
				emit(C_FN, vid, nargs);
				return;
			}
			for(size_t k = 0; k < vars_.size(); k++)
				if(vars_[k] == name) { emit(C_VAR, (int)k); return; }
			if(name == "_pi") { emit(C_NUM, 0, 3.141592653589793238462643); return; }
			if(name == "_e") { emit(C_NUM, 0, 2.718281828459045235360287); return; }
			fail("unknown variable \"" + name + "\"");
		}
		if(tok_ == T_END) fail("unexpected end");
		fail("unexpected token \"" + tv_ + "\"");
	}
};

}  // namespace nbpm
