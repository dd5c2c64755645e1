// mlp.cuh -- learned troubled-cell sensor (new component; no counterpart in the reference).
// A 64 -> 64 -> 64 -> 1 MLP with GELU hidden layers and a sigmoid output scaled to
// [0, alpha_max] replaces BlenderCalculator::get_blender and the neighbour smoothing
// (dgsem/blender_calculator.cc:123-177, dgsem/plens.cc:2926-2947) inside the RHS. Input: the
// nodal rho*p of a cell interpolated to the 4^3 GLL nodes, normalised as v/mean(v) - 1.
#pragma once

#include <cstdint>
#include <vector>

#include "device.cuh"

namespace plens_gpu {

constexpr int kMlpIn = 64, kMlpHid = 64;
constexpr int kMlpParams = kMlpHid * kMlpIn + kMlpHid + kMlpHid * kMlpHid + kMlpHid + kMlpHid + 1;

struct MlpDevice {
    float* params = nullptr;        // [kMlpParams] W1 b1 W2 b2 w3 b3
    float* params_t = nullptr;      // the same with W1, W2 transposed (CUDA-core inference kernel)
    float* params_tc = nullptr;     // W1, W2 as TF32 hi/lo tensor-core operands, then the biases
    float* tiles = nullptr;         // tensor-core form: network inputs, one 64 KB operand image per 128 cells
    float* mod = nullptr;           // tensor-core form: plain-indicator alpha of handed-back cells (-1: none)
    bool use_tc = false;            // the inference kernels with the hidden layers on the tensor cores
    const float* cbm = nullptr;     // degree 3: C1 (x) C1 (x) C1 as TF32 hi/lo operands, then its row sums
    double* alpha_plain = nullptr;  // [nc] judge: MLP alpha of the judged stage
    unsigned long long* maxerr = nullptr;  // order-preserving max per-cell alpha error
    uint8_t* mask = nullptr;        // [nc] cells handed back to the plain indicator by the judge
    unsigned int* nbad = nullptr;   // cells over the tolerance in the current judged stage
    double tol = 0.05;
    int64_t nc = 0;
    bool weights_set = false;
    int step_counter = 0;           // host-side count of steps launched (judge schedule)
    bool judge_this_step = false;
};

int mlp_create(MlpDevice& m, int64_t nc, std::vector<void*>& allocs);
int mlp_set_weights(MlpDevice& m, const float* host_params, cudaStream_t st);
// Stage-wise sensor: MLP inference (+ the plain blender on judged steps, with fallback).
int mlp_sensor_launch(MlpDevice& m, const Dev& dv, const Ops& ops, const GasP& g, const BlendP& bp, int P,
                      cudaStream_t st);
int mlp_step_begin(MlpDevice& m, const Dev& dv, int judge_every, cudaStream_t st);
int mlp_step_end(MlpDevice& m, const Dev& dv, cudaStream_t st);
// Training pairs of the current state: x [nc][64], y [nc] (plain final alpha).
int mlp_pairs(const Dev& dv, const Ops& ops, const GasP& g, const BlendP& bp, int P, float* x, float* y,
              cudaStream_t st, int64_t& launches);

}  // namespace plens_gpu
