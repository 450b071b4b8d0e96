// Host-side helpers shared by the map builder and the API.
#pragma once

#include <stdint.h>

#include "tsdfl.h"

namespace tsdfl {

constexpr int kSubTable = 64;   // sub-voxel threshold table entries (a power of two)

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
// Multiplier of the division-free sub-voxel index: for q = trunc(s / res) and
// every float s in [0, 1), returns 2 with *inv such that floor(s * inv) == q,
// else 1 with *inv such that c = floor(s * inv) is q or q - 1 and the table
// next_thr (kSubTable entries) such that q == c + (s >= next_thr[c]), else 0
// (no fast path).  next_thr[c] is the smallest float s with trunc(s / res) > c.
int sub_index_mult(float res, uint64_t sub_dim, float* inv, float* next_thr);

}  // namespace tsdfl
