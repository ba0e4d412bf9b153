// snk_particles.h -- device records and launches of the particle collision queries
// (particles.cu); layouts equal snk_particle / snk_contact of the C ABI.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

namespace snk {

struct SceneDev;

struct ParticleDev { float4 pr, vel, col; };
struct ContactOut { float n[3]; float dist; float p[3]; float pad0; float v[3]; float pad1; };
static_assert(sizeof(ParticleDev) == 48 && sizeof(ContactOut) == 48, "particle record layouts");

cudaError_t launch_contact_rays(const SceneDev& S, const float4* rays, uint32_t n, float timestep, ContactOut* out,
                                int max_blocks, cudaStream_t s);
cudaError_t launch_particle_probe(const SceneDev& S, const ParticleDev* p, uint32_t n, float timestep,
                                  ContactOut* cand, float* gravity, int max_blocks, cudaStream_t s);
cudaError_t launch_particle_constrain(const SceneDev& S, const ParticleDev* p, const float* off, uint32_t n,
                                      float timestep, float* out, int max_blocks, cudaStream_t s);

}  // namespace snk
