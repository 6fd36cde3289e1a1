// Internal definitions shared by the host C++ and CUDA translation units of
// the FDFD engine.  Nothing here is part of the public ABI.
#pragma once

#include <stdint.h>
#include <string>
#include <vector>

#include "../../include/fdfd_gb300.h"

namespace fdfd {

// Physical constants, bit-identical to fdfdpy/constants.py:3-6.
constexpr double EPSILON_0 = 8.85418782e-12;
constexpr double MU_0 = 1.25663706e-6;

// Thread-local last-error message (fdfd_last_error()).
void set_error(const std::string &msg);
int fail(int code, const std::string &msg);

// Host-side symbolic analysis (symbolic.cpp).  Arrays are host vectors;
// the factor uploads what it needs.
struct Symbolic {
    // A batch symbolic describes `batch` independent copies of one grid's
    // front tree (a forest): Nx = batch * rows rows of Ny cells, problem b
    // owning rows [b rows, (b + 1) rows) with its own periodic wrap; level L
    // holds the batch's copies of the single tree's level-L fronts.
    int32_t batch = 1, rows = 0;
    int32_t Nx = 0, Ny = 0, leaf_area = 0;
    int32_t nf = 0, nlev = 0;
    std::vector<int32_t> p, m, ld, parent, child0, child1, height, vars_off;
    std::vector<int64_t> pool_off;   // element offset of each dense front
    std::vector<int32_t> level_ptr;  // fronts of level L: [level_ptr[L], level_ptr[L+1])
    std::vector<int32_t> vars;       // per front: p pivots then m-p boundary vars
    std::vector<int32_t> relmap;     // per boundary entry: local index in parent (-1 for pivots)
    std::vector<int32_t> nbr_loc;    // 4 per cell: local index of xm,xp,ym,yp neighbour in own front or -1
    std::vector<int32_t> var_front, var_loc;
    std::vector<int32_t> lev_max_m, lev_max_p;
    int64_t sum_m = 0, pool_entries = 0, factor_entries = 0;
    double factor_flops = 0.0;
    int32_t max_m = 0, max_p = 0;
};

int build_symbolic(int32_t Nx, int32_t Ny, int32_t leaf_area, Symbolic &S);
// `batch` copies of S1 as one forest (see Symbolic::batch).
int replicate_symbolic(const Symbolic &S1, int32_t batch, Symbolic &S);

}  // namespace fdfd

// Opaque handle types of the C ABI.
struct fdfd_symbolic {
    fdfd::Symbolic s;
};
