// Host-side helpers shared by the map builder and the API.
#pragma once

#include <stdint.h>

#include "tsdfl.h"

namespace tsdfl {

void set_error(const char* fmt, ...);

uint64_t f2u_x86_host(float v);
float likelihood_value(int mm, float sigma);
float likelihood_init(float sigma);
void code_values(float sigma, float init_value, float out[604]);
void coef_init(tsdfl_map_coef* c, const float mn[3], const float mx[3], float res, float init);
uint64_t host_slot_index(const tsdfl_map_coef& c, const int32_t* grid_occ, float x, float y, float z);
// Largest trunc(offset) that passes the coarse bound check of getIndex
// (cuda_sub_voxel_map.tcc:54-66) on this axis, -1 if none.
int32_t coarse_mmax(uint64_t dim, float res);
// Multipliers of the division-free sub-voxel index q = trunc(fl(s / res)) for
// every float s in [0, 1): returns 2 with *hi such that q == floor(s * hi)
// (exact product), else 1 with (*hi, *lo) such that
// q == trunc(fl(fma(s, hi, fl(s * lo)))), else 0 (no fast path).
int sub_index_mult(float res, uint64_t sub_dim, float* hi, float* lo);

}  // namespace tsdfl
