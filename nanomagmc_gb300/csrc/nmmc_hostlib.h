// Host-side helpers of libnmmc (plain C++, no CUDA): input files, lattice masks, site
// counts, interaction-to-stencil mapping, statistics.
#pragma once

#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/nmmc.h"

namespace nmmc {

// Maps interaction records onto the 2*dim nearest-neighbour stencil directions
// (+x,-x,+y,-y,+z,-z), summing records that share an offset and skipping zero offsets.
// Records that couple anything else (any other offset with a nonzero J, or a nonzero D on a
// Heisenberg lattice) make the table "general": `general` is set and J, D are left zero; the
// records are then used as they are, in file order, by the multi-colour sweep.
int map_interactions(const nmmc_interactions& in, int dim, bool ising, double J[6], double D[6][3],
                     bool& general, std::string& why);

// Colouring of the lattice sites for a parallel Metropolis sweep with a general interaction
// table: no two sites of one colour interact through any record, so every colour class can
// be updated at once. kind 1: colour = (x + b*y + c*z) mod q (q colours); kind 2: colour =
// (x mod p) + p*(y mod p) [+ p^2*(z mod p)] (q = p^dim colours). On a periodic lattice the
// period divides the edge, so the colour is the same across the wrap.
struct Colouring {
    int kind = 0;   // 0: the two-colour checkerboard of the nearest-neighbour kernels
    int q = 2;      // number of colour classes
    int p = 2;      // kind 1: modulus q; kind 2: period p per axis
    int b = 1, c = 1;
};
int find_colouring(const nmmc_interactions& in, int dim, int edge, bool periodic, bool ising,
                   Colouring& out, std::string& why);

// Weibull shape test of Old/lib/shape.cpp:40-58 for every box site of one chain, with the
// uniform drawn from Philox (seed, chain, box index). mask: edge^dim bytes, x fastest.
void weibull_mask(int dim, int edge, double a, double wbeta, uint64_t seed, uint32_t chain,
                  uint8_t* mask);

// num / snum / s4num of Old/lib/state.cpp:124-166 for a box mask (nullptr: all filled).
void site_counts(int dim, int edge, const uint8_t* mask, int* num, int* snum, int* s4num);

// The derived edge of Old/lib/param_read.cpp:55-70 (0 for an unknown shape code).
double derived_edge(char shape, double amean, double asd);

// 2 or 3 for a known shape code, 0 otherwise (Old/lib/state.cpp:54-79).
int shape_dim(char shape);
bool shape_is_weibull(char shape);

int set_error_host(int code, const std::string& msg);

}  // namespace nmmc
