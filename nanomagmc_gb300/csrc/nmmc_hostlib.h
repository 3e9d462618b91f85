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
// Returns NMMC_ERR_UNSUPPORTED (with a message) for any other offset.
int map_interactions(const nmmc_interactions& in, int dim, double J[6], double D[6][3],
                     std::string& why);

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
