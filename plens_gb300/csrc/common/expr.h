// expr.h -- muparser-style scalar expressions in (x, y, z, t), compiled on the host into a
// stack bytecode (plens_expr_insn) and evaluated identically on the host and on the device.
//
// The reference evaluates these through deal.II's FunctionParser (muparser): the Courant number
// and wall blender limit (functions of t: dgsem/plens.cc:1489-1491, 2882-2889), the viscous
// blending region (x,y,z,t at cell centres: dgsem/plens.cc:2890-2892, 2950-2960) and the
// varying-inflow p, T and velocity (IBCs/varying_inflow.cc:17-70). Supported grammar (muparser
// precedence): ternary ?:, ||, &&, comparisons, + -, * /, unary -, ^ (right associative),
// numbers, the variables x y z t, the constants pi/_pi/_e, and the functions
// sin cos tan cot asin acos atan sinh cosh tanh exp log ln log10 log2 sqrt abs sign floor ceil
// int rint, and pow atan2 min max (min/max variadic) and if(c,a,b).
#pragma once

#include <math.h>
#include <stdint.h>

#include "plens_gpu.h"

#ifdef __CUDACC__
#define PLENS_HD __host__ __device__
#else
#define PLENS_HD
#endif

namespace plens {

enum ExprOp : int32_t {
    EOP_CONST = 0, EOP_VAR, EOP_NEG, EOP_NOT,
    EOP_ADD, EOP_SUB, EOP_MUL, EOP_DIV, EOP_POW,
    EOP_LT, EOP_GT, EOP_LE, EOP_GE, EOP_EQ, EOP_NE, EOP_AND, EOP_OR,
    EOP_JMPF, EOP_JMP,
    EOP_F1, EOP_F2
};

enum ExprFunc1 : int32_t {
    EF_SIN = 0, EF_COS, EF_TAN, EF_COT, EF_ASIN, EF_ACOS, EF_ATAN, EF_SINH, EF_COSH, EF_TANH,
    EF_EXP, EF_LOG, EF_LOG10, EF_LOG2, EF_SQRT, EF_ABS, EF_SIGN, EF_FLOOR, EF_CEIL, EF_INT,
    EF_RINT
};
enum ExprFunc2 : int32_t { EF2_POW = 0, EF2_ATAN2, EF2_MIN, EF2_MAX };

constexpr int kExprStack = 32;

PLENS_HD inline double expr_f1(int f, double a)
{
    switch (f) {
    case EF_SIN: return sin(a);
    case EF_COS: return cos(a);
    case EF_TAN: return tan(a);
    case EF_COT: return 1.0 / tan(a);
    case EF_ASIN: return asin(a);
    case EF_ACOS: return acos(a);
    case EF_ATAN: return atan(a);
    case EF_SINH: return sinh(a);
    case EF_COSH: return cosh(a);
    case EF_TANH: return tanh(a);
    case EF_EXP: return exp(a);
    case EF_LOG: return log(a);
    case EF_LOG10: return log10(a);
    case EF_LOG2: return log2(a);
    case EF_SQRT: return sqrt(a);
    case EF_ABS: return fabs(a);
    case EF_SIGN: return (a > 0) ? 1.0 : ((a < 0) ? -1.0 : 0.0);
    case EF_FLOOR: return floor(a);
    case EF_CEIL: return ceil(a);
    case EF_INT: return trunc(a);
    case EF_RINT: return rint(a);
    default: return NAN;
    }
}

PLENS_HD inline double expr_f2(int f, double a, double b)
{
    switch (f) {
    case EF2_POW: return pow(a, b);
    case EF2_ATAN2: return atan2(a, b);
    case EF2_MIN: return (a < b) ? a : b;
    case EF2_MAX: return (a > b) ? a : b;
    default: return NAN;
    }
}

// Evaluates one compiled expression. The compiler guarantees the stack depth stays below
// kExprStack; a malformed program yields NaN instead of running off the stack.
PLENS_HD inline double expr_eval(const plens_expr_insn* code, int32_t len,
                                 double x, double y, double z, double t)
{
    double st[kExprStack];
    int sp = 0;
    int pc = 0;
    int guard = 0;
    while (pc < len) {
        if (++guard > 4 * len + 16) return NAN;
        const plens_expr_insn in = code[pc];
        switch (in.op) {
        case EOP_CONST:
            if (sp >= kExprStack) return NAN;
            st[sp++] = in.val;
            break;
        case EOP_VAR: {
            if (sp >= kExprStack) return NAN;
            const double v = (in.arg == 0) ? x : (in.arg == 1) ? y : (in.arg == 2) ? z : t;
            st[sp++] = v;
            break;
        }
        case EOP_NEG: if (sp < 1) return NAN; st[sp - 1] = -st[sp - 1]; break;
        case EOP_NOT: if (sp < 1) return NAN; st[sp - 1] = (st[sp - 1] == 0.0) ? 1.0 : 0.0; break;
        case EOP_F1: if (sp < 1) return NAN; st[sp - 1] = expr_f1(in.arg, st[sp - 1]); break;
        case EOP_JMPF:
            if (sp < 1) return NAN;
            --sp;
            if (st[sp] == 0.0) { pc = in.arg; continue; }
            break;
        case EOP_JMP: pc = in.arg; continue;
        default: {
            if (sp < 2) return NAN;
            const double b = st[--sp];
            const double a = st[sp - 1];
            double r;
            switch (in.op) {
            case EOP_ADD: r = a + b; break;
            case EOP_SUB: r = a - b; break;
            case EOP_MUL: r = a * b; break;
            case EOP_DIV: r = a / b; break;
            case EOP_POW: r = pow(a, b); break;
            case EOP_LT: r = (a < b) ? 1.0 : 0.0; break;
            case EOP_GT: r = (a > b) ? 1.0 : 0.0; break;
            case EOP_LE: r = (a <= b) ? 1.0 : 0.0; break;
            case EOP_GE: r = (a >= b) ? 1.0 : 0.0; break;
            case EOP_EQ: r = (a == b) ? 1.0 : 0.0; break;
            case EOP_NE: r = (a != b) ? 1.0 : 0.0; break;
            case EOP_AND: r = (a != 0.0 && b != 0.0) ? 1.0 : 0.0; break;
            case EOP_OR: r = (a != 0.0 || b != 0.0) ? 1.0 : 0.0; break;
            case EOP_F2: r = expr_f2(in.arg, a, b); break;
            default: return NAN;
            }
            st[sp - 1] = r;
            break;
        }
        }
        ++pc;
    }
    return (sp == 1) ? st[0] : NAN;
}

PLENS_HD inline double expr_eval_table(const plens_params& prm, const plens_expr_insn* code,
                                       int32_t idx, double x, double y, double z, double t)
{
    if (idx < 0 || idx >= prm.n_expr) return NAN;
    return expr_eval(code + prm.expr_offset[idx], prm.expr_length[idx], x, y, z, t);
}

}  // namespace plens
