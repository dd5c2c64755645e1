// expr_compile.h -- host-side compiler for the expression bytecode of common/expr.h.
#pragma once

#include <string>
#include <vector>

#include "plens_gpu.h"

namespace plens {

// A table of compiled expressions sharing one instruction array, in the layout plens_params
// carries (expr_offset / expr_length / expr_code).
struct ExprTable {
    std::vector<int32_t> offset, length;
    std::vector<plens_expr_insn> code;

    // Compiles `src` and returns its index; throws std::runtime_error with a message that names
    // the expression and the position of the first error.
    int32_t add(const std::string& src);
    double eval(int32_t idx, double x, double y, double z, double t) const;
    int32_t size() const { return static_cast<int32_t>(offset.size()); }
};

// Compiles one expression to bytecode (appended to `out`); throws on a syntax error.
void compile_expression(const std::string& src, std::vector<plens_expr_insn>& out);

}  // namespace plens
