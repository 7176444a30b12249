// ORACLE — test infrastructure only. The reference's shared shader functions
// (shader/rand.hlsl, enc.inc.hlsl, gbuffer.hlsl, restir/reservoir.hlsl,
// restir/hash_grid.inc.hlsl), compiled from their own text, behind a C ABI for
// known-answer comparisons with the oracle restatement.
#include "hlsl.hpp"
#include "vlt.h"

namespace hlsl {
namespace ref_primitives {
#include "shader/rand.hlsl"
#include "shader/enc.inc.hlsl"
#include "shader/gbuffer.hlsl"
#include "shader/restir/reservoir.hlsl"
#include "shader/restir/hash_grid.inc.hlsl"
}  // namespace ref_primitives
}  // namespace hlsl

using namespace hlsl;
namespace P = hlsl::ref_primitives;

extern "C" {

void vltr_jenkins_hash(const uint32_t* x, uint32_t* out, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) out[i] = P::jenkins_hash(x[i]);
}

// lcg_init_with_seed(pixel, seed), then `count` lcg_rand draws: floats and states.
void vltr_lcg_sequence(uint32_t px, uint32_t py, uint32_t seed, uint32_t count, float* rands, uint32_t* states) {
  uint32_t s = P::lcg_init_with_seed(uint2(px, py), seed);
  for (uint32_t k = 0; k < count; ++k) {
    rands[k] = P::lcg_rand(s);
    states[k] = s;
  }
}

uint32_t vltr_xxhash32(const uint32_t* words, uint32_t n) {
  P::XXHash32 h = P::XXHash32::init(words[0]);
  for (uint32_t i = 1; i < n; ++i) h = h.add(words[i]);
  return h.eval();
}

void vltr_oct_encode(const float* n3, uint32_t* u16, uint32_t* u32, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    float3 v(n3[3 * i], n3[3 * i + 1], n3[3 * i + 2]);
    u16[i] = P::normal_encode_oct_u16(v);
    u32[i] = P::normal_encode_oct_u32(v);
  }
}

void vltr_oct_decode(const uint32_t* u16, const uint32_t* u32, float* n16, float* n32, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    float3 a = P::normal_decode_oct_u16(u16[i]);
    float3 b = P::normal_decode_oct_u32(u32[i]);
    for (int k = 0; k < 3; ++k) {
      n16[3 * i + k] = a.e[k];
      n32[3 * i + k] = b.e[k];
    }
  }
}

void vltr_reservoir_simple(const uint32_t* M, const float* W, uint32_t* enc, uint32_t* dec_M, float* dec_W,
                           uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    P::ReservoirSimple r = {M[i], W[i]};
    enc[i] = r.encode_32b();
    P::ReservoirSimple d = P::ReservoirSimple::decode_32b(enc[i]);
    dec_M[i] = d.M;
    dec_W[i] = d.W;
  }
}

// HitPosNormal::encode of (pos, normal), then decode of the encoding.
void vltr_hit_pos_normal(const float* pos, const float* nrm, uint32_t* enc, float* dec_pos, float* dec_nrm,
                         uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    P::HitPosNormal h = {float3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]),
                         float3(nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2])};
    uint2 e = h.encode();
    enc[2 * i] = e.e[0];
    enc[2 * i + 1] = e.e[1];
    P::HitPosNormal d = P::HitPosNormal::decode(e);
    for (int k = 0; k < 3; ++k) {
      dec_pos[3 * i + k] = d.pos.e[k];
      dec_nrm[3 * i + k] = d.normal.e[k];
    }
  }
}

// VertexDescriptor::create(pos, dir) with frame_params.view_pos = camera; out:
// {hash, checksum, lod, pos_packed.x, pos_packed.y} per point.
void vltr_vertex_key(const float* pos, const float* camera, uint32_t* out, uint32_t n) {
  P::frame_params.view_pos = float4(camera[0], camera[1], camera[2], 1.0f);
  for (uint32_t i = 0; i < n; ++i) {
    P::VertexDescriptor v = P::VertexDescriptor::create(float3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]),
                                                        float3(0.0f, 0.0f, 1.0f));
    out[5 * i + 0] = v.hash();
    out[5 * i + 1] = v.checksum();
    out[5 * i + 2] = v.lod;
    out[5 * i + 3] = v.pos_packed.e[0];
    out[5 * i + 4] = v.pos_packed.e[1];
  }
}

// decode_gbuffer of 4-word texels: {color.rgb, metallic, normal.xyz, roughness,
// fwidth_z, fwidth_n, shading_path (as float bits)} per texel.
void vltr_gbuffer_decode(const uint32_t* enc, float* out, uint32_t n) {
  for (uint32_t i = 0; i < n; ++i) {
    P::GBuffer g = P::decode_gbuffer(uint4(enc[4 * i], enc[4 * i + 1], enc[4 * i + 2], enc[4 * i + 3]));
    float* o = out + 11 * i;
    for (int k = 0; k < 3; ++k) o[k] = g.color.e[k];
    o[3] = g.metallic;
    for (int k = 0; k < 3; ++k) o[4 + k] = g.normal.e[k];
    o[7] = g.perceptual_roughness;
    o[8] = g.fwidth_z;
    o[9] = g.fwidth_n;
    o[10] = orc::asfloat(g.shading_path);
  }
}

}  // extern "C"
