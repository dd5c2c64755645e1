// expr_compile.cpp -- recursive-descent compiler from muparser-style infix expressions to the
// stack bytecode of common/expr.h. Stands in for deal.II's FunctionParser, which the reference
// uses for every run-time expression (see common/expr.h for the call sites).
#include "expr_compile.h"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <map>
#include <stdexcept>

#include "../common/expr.h"

namespace plens {

namespace {

struct Parser {
    const std::string& s;
    size_t pos = 0;
    std::vector<plens_expr_insn> code;
    int depth = 0, max_depth = 0;

    explicit Parser(const std::string& src) : s(src) {}

    [[noreturn]] void fail(const std::string& what) const
    {
        throw std::runtime_error("expression '" + s + "': " + what + " at position " +
                                 std::to_string(pos));
    }
    void skip()
    {
        while (pos < s.size() && std::isspace(static_cast<unsigned char>(s[pos]))) ++pos;
    }
    bool peek(const char* tok)
    {
        skip();
        return s.compare(pos, std::char_traits<char>::length(tok), tok) == 0;
    }
    bool accept(const char* tok)
    {
        if (peek(tok)) {
            pos += std::char_traits<char>::length(tok);
            return true;
        }
        return false;
    }
    void expect(const char* tok)
    {
        if (!accept(tok)) fail(std::string("expected '") + tok + "'");
    }
    void emit(int32_t op, int32_t arg = 0, double val = 0.0, int stack_delta = 0)
    {
        code.push_back(plens_expr_insn{op, arg, val});
        depth += stack_delta;
        if (depth > max_depth) max_depth = depth;
    }

    // ternary := or ( '?' ternary ':' ternary )?
    void ternary()
    {
        logic_or();
        if (accept("?")) {
            const size_t jf = code.size();
            emit(EOP_JMPF, 0, 0, -1);
            ternary();
            const size_t jend = code.size();
            emit(EOP_JMP, 0, 0, 0);
            depth -= 1;  // the else branch pushes in place of the then branch
            code[jf].arg = static_cast<int32_t>(code.size());
            expect(":");
            ternary();
            code[jend].arg = static_cast<int32_t>(code.size());
        }
    }
    void logic_or()
    {
        logic_and();
        while (accept("||")) { logic_and(); emit(EOP_OR, 0, 0, -1); }
    }
    void logic_and()
    {
        comparison();
        while (accept("&&")) { comparison(); emit(EOP_AND, 0, 0, -1); }
    }
    void comparison()
    {
        additive();
        for (;;) {
            int32_t op;
            if (accept("<=")) op = EOP_LE;
            else if (accept(">=")) op = EOP_GE;
            else if (accept("==")) op = EOP_EQ;
            else if (accept("!=")) op = EOP_NE;
            else if (accept("<")) op = EOP_LT;
            else if (accept(">")) op = EOP_GT;
            else break;
            additive();
            emit(op, 0, 0, -1);
        }
    }
    void additive()
    {
        multiplicative();
        for (;;) {
            if (accept("+")) { multiplicative(); emit(EOP_ADD, 0, 0, -1); }
            else if (accept("-")) { multiplicative(); emit(EOP_SUB, 0, 0, -1); }
            else break;
        }
    }
    void multiplicative()
    {
        unary();
        for (;;) {
            if (accept("*")) { unary(); emit(EOP_MUL, 0, 0, -1); }
            else if (accept("/")) { unary(); emit(EOP_DIV, 0, 0, -1); }
            else break;
        }
    }
    // unary minus binds weaker than ^ (muparser: -2^2 = -4)
    void unary()
    {
        if (accept("-")) { unary(); emit(EOP_NEG); return; }
        if (accept("+")) { unary(); return; }
        if (peek("!") && !peek("!=")) { ++pos; unary(); emit(EOP_NOT); return; }
        power();
    }
    void power()
    {
        primary();
        if (accept("^")) {
            unary();  // right associative, allows 2^-1
            emit(EOP_POW, 0, 0, -1);
        }
    }
    void primary()
    {
        skip();
        if (pos >= s.size()) fail("unexpected end");
        const char c = s[pos];
        if (std::isdigit(static_cast<unsigned char>(c)) || c == '.') {
            const char* begin = s.c_str() + pos;
            char* end = nullptr;
            const double v = std::strtod(begin, &end);
            if (end == begin) fail("bad number");
            pos += static_cast<size_t>(end - begin);
            emit(EOP_CONST, 0, v, +1);
            return;
        }
        if (accept("(")) {
            ternary();
            expect(")");
            return;
        }
        if (std::isalpha(static_cast<unsigned char>(c)) || c == '_') {
            size_t e = pos;
            while (e < s.size() &&
                   (std::isalnum(static_cast<unsigned char>(s[e])) || s[e] == '_'))
                ++e;
            const std::string id = s.substr(pos, e - pos);
            pos = e;
            static const std::map<std::string, int32_t> vars = {
                {"x", 0}, {"y", 1}, {"z", 2}, {"t", 3}};
            static const std::map<std::string, double> consts = {
                {"pi", M_PI}, {"_pi", M_PI}, {"_e", M_E}};
            static const std::map<std::string, int32_t> f1 = {
                {"sin", EF_SIN},   {"cos", EF_COS},     {"tan", EF_TAN},   {"cot", EF_COT},
                {"asin", EF_ASIN}, {"acos", EF_ACOS},   {"atan", EF_ATAN}, {"sinh", EF_SINH},
                {"cosh", EF_COSH}, {"tanh", EF_TANH},   {"exp", EF_EXP},   {"log", EF_LOG},
                {"ln", EF_LOG},    {"log10", EF_LOG10}, {"log2", EF_LOG2}, {"sqrt", EF_SQRT},
                {"abs", EF_ABS},   {"sign", EF_SIGN},   {"floor", EF_FLOOR},
                {"ceil", EF_CEIL}, {"int", EF_INT},     {"rint", EF_RINT}};
            static const std::map<std::string, int32_t> f2 = {
                {"pow", EF2_POW}, {"atan2", EF2_ATAN2}, {"min", EF2_MIN}, {"max", EF2_MAX}};
            auto v = vars.find(id);
            if (v != vars.end()) { emit(EOP_VAR, v->second, 0, +1); return; }
            auto k = consts.find(id);
            if (k != consts.end()) { emit(EOP_CONST, 0, k->second, +1); return; }
            auto g1 = f1.find(id);
            if (g1 != f1.end()) {
                expect("(");
                ternary();
                expect(")");
                emit(EOP_F1, g1->second);
                return;
            }
            auto g2 = f2.find(id);
            if (g2 != f2.end()) {
                expect("(");
                ternary();
                int nargs = 1;
                while (accept(",")) {
                    ternary();
                    ++nargs;
                    if (g2->second == EF2_MIN || g2->second == EF2_MAX)
                        emit(EOP_F2, g2->second, 0, -1);  // fold variadic min/max
                }
                expect(")");
                if (g2->second == EF2_MIN || g2->second == EF2_MAX) {
                    if (nargs < 1) fail("min/max need an argument");
                } else {
                    if (nargs != 2) fail(id + " takes two arguments");
                    emit(EOP_F2, g2->second, 0, -1);
                }
                return;
            }
            if (id == "if") {
                expect("(");
                ternary();
                const size_t jf = code.size();
                emit(EOP_JMPF, 0, 0, -1);
                expect(",");
                ternary();
                const size_t jend = code.size();
                emit(EOP_JMP);
                depth -= 1;
                code[jf].arg = static_cast<int32_t>(code.size());
                expect(",");
                ternary();
                code[jend].arg = static_cast<int32_t>(code.size());
                expect(")");
                return;
            }
            fail("unknown identifier '" + id + "'");
        }
        fail(std::string("unexpected character '") + c + "'");
    }
};

}  // namespace

void compile_expression(const std::string& src, std::vector<plens_expr_insn>& out)
{
    Parser p(src);
    p.ternary();
    p.skip();
    if (p.pos != src.size()) p.fail("trailing input");
    if (p.max_depth >= kExprStack) p.fail("expression too deep");
    // jump targets are relative to the expression start; the table keeps them that way
    out.insert(out.end(), p.code.begin(), p.code.end());
}

int32_t ExprTable::add(const std::string& src)
{
    std::vector<plens_expr_insn> prog;
    compile_expression(src, prog);
    offset.push_back(static_cast<int32_t>(code.size()));
    length.push_back(static_cast<int32_t>(prog.size()));
    code.insert(code.end(), prog.begin(), prog.end());
    return static_cast<int32_t>(offset.size()) - 1;
}

double ExprTable::eval(int32_t idx, double x, double y, double z, double t) const
{
    if (idx < 0 || idx >= size()) return NAN;
    return expr_eval(code.data() + offset[idx], length[idx], x, y, z, t);
}

}  // namespace plens
