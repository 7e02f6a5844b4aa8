// The particle file of BaseSpecies::save / load (src/particles.cpp:32-93):
//   int32 total slots, int32 live particles, then one 64-byte t_particle
//   record per live particle (src/particles.hpp:26-33): doubles x, y, z, vx,
//   vy, vz, time_to_death, a bool empty (false) and 7 bytes of padding;
//   little-endian, as the reference writes its in-memory structs on x86-64
//   and aarch64.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace mag {

struct ParticleFile {
    int32_t total = 0;  // slots of the writing species (live + free)
    std::vector<double> x, y, z, vx, vy, vz, ttd;
};

ParticleFile read_particle_file(const std::string& path);
void write_particle_file(const std::string& path, const ParticleFile& f);
// the source box file (int32 count, then records); false when it cannot be opened
bool read_source_file(const std::string& path, ParticleFile& f);
void write_source_file(const std::string& path, const ParticleFile& f);

}  // namespace mag
