// The custom excitation signal: an expression of the time t in the syntax of
// the function parser openEMS hands it to (Excitation::CalcCustomExcitation,
// excitation.cpp:233-271: constants pi and e, variable t), compiled once to
// a postfix program and evaluated in double for every sample.
//
// Covered: numbers, t, pi, e, + - * / % ^ (power, right-associative, above
// unary minus: -t^2 = -(t^2)), parentheses and the functions abs acos acosh
// asin asinh atan atanh cbrt ceil cos cosh exp exp2 floor int (nearest
// integer) log log10 log2 sin sinh sqrt tan tanh trunc (one argument) and
// atan2 hypot max min pow (two).  Comparisons, logical operators and if()
// carry the parser's own truth conventions and are refused.
#pragma once

#include <cctype>
#include <cmath>
#include <string>
#include <vector>

namespace wipems {

class SignalExpr {
public:
    // false with a message on a syntax error or an unsupported construct
    bool compile(const std::string& text, std::string& err) {
        src_ = text;
        pos_ = 0;
        prog_.clear();
        err_.clear();
        if (!expr()) {
            err = err_;
            return false;
        }
        skip();
        if (pos_ != src_.size()) {
            err = "unexpected '" + src_.substr(pos_, 1) + "' at position " + std::to_string(pos_);
            return false;
        }
        return true;
    }

    double eval(double t) const {
        std::vector<double> st;
        st.reserve(16);
        for (const Ins& in : prog_) {
            double b, a;
            switch (in.op) {
                case OP_NUM: st.push_back(in.v); break;
                case OP_T: st.push_back(t); break;
                case OP_NEG: st.back() = -st.back(); break;
                case OP_FN1: st.back() = fn1(in.fn, st.back()); break;
                default:
                    b = st.back();
                    st.pop_back();
                    a = st.back();
                    st.back() = bin(in.op, in.fn, a, b);
                    break;
            }
        }
        return st.empty() ? 0.0 : st.back();
    }

private:
    enum Op { OP_NUM, OP_T, OP_NEG, OP_FN1, OP_ADD, OP_SUB, OP_MUL, OP_DIV, OP_MOD, OP_POW, OP_FN2 };
    struct Ins {
        Op op;
        int fn;
        double v;
    };
    std::string src_, err_;
    size_t pos_ = 0;
    std::vector<Ins> prog_;

    static const char* const* names1() {
        static const char* const n[] = {"abs",  "acos", "acosh", "asin", "asinh", "atan",  "atanh", "cbrt",
                                        "ceil", "cos",  "cosh",  "exp",  "exp2",  "floor", "int",   "log",
                                        "log10", "log2", "sin",  "sinh", "sqrt",  "tan",   "tanh",  "trunc", nullptr};
        return n;
    }
    static const char* const* names2() {
        static const char* const n[] = {"atan2", "hypot", "max", "min", "pow", nullptr};
        return n;
    }
    static double fn1(int f, double x) {
        switch (f) {
            case 0: return std::fabs(x);
            case 1: return std::acos(x);
            case 2: return std::acosh(x);
            case 3: return std::asin(x);
            case 4: return std::asinh(x);
            case 5: return std::atan(x);
            case 6: return std::atanh(x);
            case 7: return std::cbrt(x);
            case 8: return std::ceil(x);
            case 9: return std::cos(x);
            case 10: return std::cosh(x);
            case 11: return std::exp(x);
            case 12: return std::exp2(x);
            case 13: return std::floor(x);
            case 14: return std::floor(x + 0.5);
            case 15: return std::log(x);
            case 16: return std::log10(x);
            case 17: return std::log2(x);
            case 18: return std::sin(x);
            case 19: return std::sinh(x);
            case 20: return std::sqrt(x);
            case 21: return std::tan(x);
            case 22: return std::tanh(x);
            default: return std::trunc(x);
        }
    }
    static double bin(int op, int f, double a, double b) {
        switch (op) {
            case OP_ADD: return a + b;
            case OP_SUB: return a - b;
            case OP_MUL: return a * b;
            case OP_DIV: return a / b;
            case OP_MOD: return std::fmod(a, b);
            case OP_POW: return std::pow(a, b);
            default:
                switch (f) {
                    case 0: return std::atan2(a, b);
                    case 1: return std::hypot(a, b);
                    case 2: return a > b ? a : b;
                    case 3: return a < b ? a : b;
                    default: return std::pow(a, b);
                }
        }
    }

    void skip() {
        while (pos_ < src_.size() && std::isspace((unsigned char)src_[pos_])) ++pos_;
    }
    bool take(char c) {
        skip();
        if (pos_ < src_.size() && src_[pos_] == c) {
            ++pos_;
            return true;
        }
        return false;
    }
    bool fail(const std::string& m) {
        if (err_.empty()) err_ = m;
        return false;
    }
    void emit(Op op, int fn = 0, double v = 0) { prog_.push_back(Ins{op, fn, v}); }

    bool expr() {  // term (('+'|'-') term)*
        if (!term()) return false;
        for (;;) {
            if (take('+')) {
                if (!term()) return false;
                emit(OP_ADD);
            } else if (take('-')) {
                if (!term()) return false;
                emit(OP_SUB);
            } else {
                return true;
            }
        }
    }
    bool term() {  // unary (('*'|'/'|'%') unary)*
        if (!unary()) return false;
        for (;;) {
            if (take('*')) {
                if (!unary()) return false;
                emit(OP_MUL);
            } else if (take('/')) {
                if (!unary()) return false;
                emit(OP_DIV);
            } else if (take('%')) {
                if (!unary()) return false;
                emit(OP_MOD);
            } else {
                return true;
            }
        }
    }
    bool unary() {  // '-' unary | power
        if (take('-')) {
            if (!unary()) return false;
            emit(OP_NEG);
            return true;
        }
        return power();
    }
    bool power() {  // primary ('^' unary)?
        if (!primary()) return false;
        if (take('^')) {
            if (!unary()) return false;
            emit(OP_POW);
        }
        return true;
    }
    bool primary() {
        skip();
        if (pos_ >= src_.size()) return fail("expression ends early");
        const char c = src_[pos_];
        if (take('(')) {
            if (!expr()) return false;
            return take(')') ? true : fail("missing ')'");
        }
        if (std::isdigit((unsigned char)c) || c == '.') {
            const char* b = src_.c_str() + pos_;
            char* end = nullptr;
            const double v = std::strtod(b, &end);
            if (end == b) return fail("bad number at position " + std::to_string(pos_));
            pos_ += (size_t)(end - b);
            emit(OP_NUM, 0, v);
            return true;
        }
        if (std::isalpha((unsigned char)c) || c == '_') {
            size_t e = pos_;
            while (e < src_.size() && (std::isalnum((unsigned char)src_[e]) || src_[e] == '_')) ++e;
            const std::string id = src_.substr(pos_, e - pos_);
            pos_ = e;
            if (id == "t") return emit(OP_T), true;
            if (id == "pi") return emit(OP_NUM, 0, 3.14159265358979323846), true;
            if (id == "e") return emit(OP_NUM, 0, 2.71828182845904523536), true;
            for (int k = 0; names1()[k]; ++k)
                if (id == names1()[k]) {
                    if (!take('(') || !expr() || !take(')')) return fail("bad call of " + id + "()");
                    emit(OP_FN1, k);
                    return true;
                }
            for (int k = 0; names2()[k]; ++k)
                if (id == names2()[k]) {
                    if (!take('(') || !expr() || !take(',') || !expr() || !take(')'))
                        return fail("bad call of " + id + "(a, b)");
                    emit(OP_FN2, k);
                    return true;
                }
            return fail("unknown name '" + id + "' (the variable is t; constants pi, e)");
        }
        return fail(std::string("unsupported '") + c + "' at position " + std::to_string(pos_));
    }
};

}  // namespace wipems
