// ORACLE — test infrastructure only. Binary64 replay of the float storage forms'
// lighting back end (oracle64r.cpp), driven by oracle.cpp's frame driver.
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <vector>

#include "../include/vlt.h"

constexpr int R64_TAPE_WORDS = 128;  // decision-tape words per pixel and pass

struct R64;
R64* r64_create(int w, int h, const vlt_params& p);
void r64_destroy(R64* r);
void r64_ao_gen(R64& R, const vlt_frame_params& fp, const uint32_t* hpn, const float* depth, uint32_t has_new,
                uint32_t has_prev, float radius, const uint16_t* tape);
void r64_ao_filter(R64& R, const float* depth, const uint16_t* tape);
void r64_diff_temporal(R64& R, const vlt_frame_params& fp, const float* prev_depth, const float* depth,
                       const uint32_t* new_hpn, const uint32_t* new_rad, const float* new_pdf, uint32_t frame_rand,
                       uint32_t has_prev, uint32_t has_new, const uint16_t* tape);
void r64_diff_spatial(R64& R, const vlt_frame_params& fp, const uint32_t* gbuf, const float* depth,
                      uint32_t frame_rand, bool last, const uint16_t* tape);
void r64_diff_commit(R64& R);
void r64_spec_temporal(R64& R, const vlt_frame_params& fp, const float* prev_depth, const uint32_t* prev_gbuf,
                       const float* depth, const uint32_t* gbuf, const float* new_hp, const uint32_t* new_rad,
                       uint32_t frame_rand, uint32_t has_prev, const uint16_t* tape);
void r64_spec_commit(R64& R);
void r64_spec_spatial(R64& R, const vlt_frame_params& fp, const uint32_t* gbuf, const float* depth,
                      uint32_t frame_rand, bool last, const uint16_t* tape);
void r64_denoise(R64& R, const vlt_frame_params& fp, const float* depth, const uint32_t* gbuf,
                 const float* prev_depth, const uint32_t* prev_gbuf, uint32_t has_history, const uint16_t* tape);
uint64_t r64_take_flips();
// Flips of the last frame per pass: AO generation, AO filter, diffuse temporal,
// diffuse spatial, specular temporal, specular spatial, denoiser.
#define R64_FLIP_PASSES 7
void r64_take_flips_by_pass(uint64_t* out);
const double* r64_buffer(R64& R, const char* name, size_t* per_pixel, std::vector<double>& scratch);
