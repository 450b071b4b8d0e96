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
// Threshold table of the division-free sub-voxel index (MapView::sub_thr):
// thr[k] = smallest float s >= 0 with trunc(s / res) >= k (2.0 when none below
// 2), and a multiplier inv with floor(s * inv) in {q - 1, q} for q = trunc(s / res)
// and every float s in [0, 1).  Returns 0 when no such table fits in n entries,
// 2 when inv alone is exact (floor(s * inv) == q for every such s), else 1.
int sub_index_table(float res, uint64_t sub_dim, float* inv, float* thr, int n);

}  // namespace tsdfl
