// BaseSpecies::save / load file format (particle_io.hpp).
#include "particle_io.hpp"

#include <algorithm>
#include <cstring>
#include <fstream>

#include "host_config.hpp"

namespace mag {

namespace {
constexpr size_t kRecord = 64;  // sizeof(t_particle): 7 doubles, bool, padding
static_assert(sizeof(double) == 8, "t_particle layout");
}  // namespace

ParticleFile read_particle_file(const std::string& path)
{
    std::ifstream fr(path, std::ios::in | std::ios::binary);
    if (!fr.is_open()) throw Error(-6, "Species::load(): failed opening file");
    ParticleFile f;
    int32_t n = 0;
    fr.read((char*)&f.total, 4);
    fr.read((char*)&n, 4);
    if (!fr.good() || n < 0 || f.total < n) throw Error(-1, "Species::load(): inconsistent header in " + path);
    for (auto* v : {&f.x, &f.y, &f.z, &f.vx, &f.vy, &f.vz, &f.ttd}) v->resize(n);
    unsigned char rec[kRecord];
    for (int32_t i = 0; i < n; ++i) {
        fr.read((char*)rec, kRecord);
        if (!fr.good()) throw Error(-1, "Species::load(): read error in " + path);
        double d[7];
        std::memcpy(d, rec, sizeof d);
        f.x[i] = d[0];
        f.y[i] = d[1];
        f.z[i] = d[2];
        f.vx[i] = d[3];
        f.vy[i] = d[4];
        f.vz[i] = d[5];
        f.ttd[i] = d[6];
    }
    return f;
}

// BaseSpecies::source5_save / source5_load (src/particles.cpp:109-140): an
// int32 count, then the records; no total/live pair
static void read_records(std::ifstream& fr, int32_t n, ParticleFile& f, const std::string& path)
{
    for (auto* v : {&f.x, &f.y, &f.z, &f.vx, &f.vy, &f.vz, &f.ttd}) v->resize(n);
    unsigned char rec[kRecord];
    for (int32_t i = 0; i < n; ++i) {
        fr.read((char*)rec, kRecord);
        if (!fr.good()) throw Error(-1, "Species::source5_load(): read error in " + path);
        double d[7];
        std::memcpy(d, rec, sizeof d);
        f.x[i] = d[0];
        f.y[i] = d[1];
        f.z[i] = d[2];
        f.vx[i] = d[3];
        f.vy[i] = d[4];
        f.vz[i] = d[5];
        f.ttd[i] = d[6];
    }
}

bool read_source_file(const std::string& path, ParticleFile& f)
{
    std::ifstream fr(path, std::ios::in | std::ios::binary);
    if (!fr.is_open()) return false;  // the reference warns and keeps its source particles
    int32_t n = 0;
    fr.read((char*)&n, 4);
    if (!fr.good() || n < 0) throw Error(-1, "Species::source5_load(): bad header in " + path);
    f.total = n;
    read_records(fr, n, f, path);
    return true;
}

void write_source_file(const std::string& path, const ParticleFile& f)
{
    std::ofstream fw(path, std::ios::out | std::ios::binary);
    if (!fw.is_open()) throw Error(-6, "Species::source_save(): failed opening file");
    const int32_t n = (int32_t)f.x.size();
    fw.write((const char*)&n, 4);
    unsigned char rec[kRecord];
    for (int32_t i = 0; i < n; ++i) {
        std::memset(rec, 0, kRecord);
        const double d[7] = {f.x[i], f.y.empty() ? 0.0 : f.y[i], f.z[i], f.vx[i], f.vy[i], f.vz[i],
                             f.ttd.empty() ? 0.0 : f.ttd[i]};
        std::memcpy(rec, d, sizeof d);
        fw.write((const char*)rec, kRecord);
    }
    if (!fw.good()) throw Error(-1, "Species::source_save(): write error in " + path);
}

void write_particle_file(const std::string& path, const ParticleFile& f)
{
    std::ofstream fw(path, std::ios::out | std::ios::binary);
    if (!fw.is_open()) throw Error(-6, "Species::save(): failed opening file");
    const int32_t n = (int32_t)f.x.size();
    const int32_t total = std::max(f.total, n);
    fw.write((const char*)&total, 4);
    fw.write((const char*)&n, 4);
    unsigned char rec[kRecord];
    for (int32_t i = 0; i < n; ++i) {
        std::memset(rec, 0, kRecord);
        const double d[7] = {f.x[i], f.y.empty() ? 0.0 : f.y[i], f.z[i], f.vx[i], f.vy[i], f.vz[i],
                             f.ttd.empty() ? 0.0 : f.ttd[i]};
        std::memcpy(rec, d, sizeof d);  // empty = false (0), padding zero
        fw.write((const char*)rec, kRecord);
    }
    if (!fw.good()) throw Error(-1, "Species::save(): write error in " + path);
}

}  // namespace mag
