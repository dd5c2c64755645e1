// main.cpp -- command-line entry, as the reference's main.cc:41-108:
//   plens_gpu.out <mapping degree> <fe degree>      (reads ./input.prm)
#include <cstdio>
#include <cstdlib>
#include <exception>

#include "plens_driver.h"

int main(int argc, char** argv)
{
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s <mapping degree> <fe degree>\n", argv[0]);
        return 1;
    }
    try {
        plens::PLENS problem(std::atoi(argv[1]), std::atoi(argv[2]));
        problem.read_mesh();
        problem.set_NS();
        problem.set_dof_handler();
        problem.set_sol_vecs();
        problem.set_IC();
        problem.set_BC();
        problem.set_blender();
        problem.read_time_settings();
        problem.run();
    } catch (const std::exception& e) {
        std::fprintf(stderr, "%s\n", e.what());
        return 1;
    }
    return 0;
}
