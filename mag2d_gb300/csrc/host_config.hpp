// Host-side inputs of the PIC step: config.txt (Param), species_conf
// (SpeciesParams / InteractionParams) and the electrode geometry (t_grid).
#pragma once

#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "device.hpp"

namespace mag {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// Physical constants of the reference (src/param.cpp:6-11), kept verbatim.
constexpr double kEps0 = 8.854187817e-12;
constexpr double kKB = 1.380662e-23;
constexpr double kQe = 1.602189e-19;

// key = value configuration reader with the GetPot conventions the reference's
// config files rely on: '#' comments, [section] prefixes, ${op a b} arithmetic,
// integers read through double.
class KeyValueConfig {
public:
    KeyValueConfig() = default;
    static KeyValueConfig from_file(const std::string& path);
    static KeyValueConfig from_text(const std::string& text);
    void set(const std::string& key, const std::string& value) { vars_[key] = value; }
    bool has(const std::string& key) const { return vars_.count(key) != 0; }
    double get(const std::string& key, double dflt) const;
    int get(const std::string& key, int dflt) const { return (int)get(key, (double)dflt); }
    std::string get(const std::string& key, const char* dflt) const;

private:
    std::map<std::string, std::string> vars_;
    void parse(const std::string& text);
    std::string expand(const std::string& in, const std::string& section) const;
};

enum Coord { CARTESIAN = 0, CYLINDRICAL = 1, CARTESIAN3D = 2 };
enum Boundary { BND_FREE = 0, BND_PERIODIC = 1, BND_MIRROR = 2 };
// the movers Param accepts (param.cpp:97-105; its ADVANCE_LEAPFROG cannot be selected)
enum Mover { ADVANCE_BORIS = 0, ADVANCE_MULTICOLL = 1 };
enum Geometry {
    GEO_EMPTY, GEO_PROBE, GEO_RF_22PT, GEO_RF_8PT, GEO_RF_HAITRAP, GEO_RF_QUAD, GEO_MAC,
    GEO_PENNING, GEO_PENNING_SIMPLE, GEO_TUBE,
    GEO_PENNING_ENDCAP  // added: end caps + (segmented) ring of an orthogonal Penning trap
};

// Param (src/param.hpp:17-82, src/param.cpp:12-143)
struct Param {
    double x_max, y_max, z_max, x_min = 0, y_min = 0, z_min = 0;
    int x_sampl, y_sampl, z_sampl;
    double n_particles_total, density_total, pressure, neutral_temperature;
    double probe_radius, probe_length, u_probe, extern_field;
    std::string electric_field_static_file, electric_field_rf_file, magnetic_field_file;
    bool electric_field_from_file, has_probe, magnetic_field_const;
    double Br, Bz, Bt;
    uint64_t niter;
    double dt_elon;
    bool selfconsistent, use_source, u_smooth, rf;
    double rf_amplitude, rf_U0, rf_omega;
    uint64_t t_print, t_print_dist, t_dist_sample, t_equilib;
    bool particle_reload;
    std::string particle_reload_dir;
    int src_fact;
    double neutral_density;
    bool do_plot;
    Coord coord;
    Boundary boundary;
    Mover mover;
    Geometry geometry;
    double macroparticle_factor;
    double dx, dz, idx, idz, V, dV, dy, idy;
    // PENNING_ENDCAP geometry (no reference counterpart)
    double u_endcap, u_ring;
    std::vector<double> u_segments;
};

Param make_param(const KeyValueConfig& cfg);

enum SpeciesType { NEUTRAL = 0, ELECTRON = 1, ION = 2 };

// src/parser.hpp:16-41; values the reference leaves unset read as 0 here
struct SpeciesParams {
    std::string name;
    SpeciesType type = NEUTRAL;
    double charge = 0, mass = 0, dt = 0, density = 0, temperature = 0, polarizability = 0, E_max = 0;
};
struct InteractionParams {
    std::string name;
    CollType type = ELASTIC;
    double DE = 0, rate = 0, cutoff = 0;
    std::string primary, secondary;
    std::vector<double> CS_energy, CS_value;
};

// config_parse (src/parser.cpp:25-147)
void parse_species_conf(const std::string& path, std::vector<SpeciesParams>& species,
                        std::vector<InteractionParams>& interactions);

// Interaction::sigma_v (src/particles.hpp:61-70) for interaction 'in' of
// species prim with species sec; in.rate is the effective rate (LANGEVIN
// rates already multiplied by cutoff^2 as in particles.hpp:81-82).
double interaction_sigma_v(const InteractionParams& in, const std::vector<SpeciesParams>& sp, int prim, int sec,
                           double v);
// Null-collision rates of species s against every species and its lifetime
// (BaseSpecies::lifetime_init / svmax_find, src/particles.cpp:142-206).
// 'inters' are the parsed interactions (LANGEVIN scaling applied here).
void species_rates(const std::vector<SpeciesParams>& sp, const std::vector<InteractionParams>& inters, int s,
                   std::vector<double>& rates, double& lifetime);

// t_grid (src/fields.cpp:374-868): mask and voltage, row-major [i*z_sampl + j]
enum MaskType : int8_t { FIXED = 0, FIXED_RF = 1, FREE = 2, BOUNDARY = 3 };
void build_geometry(const Param& p, std::vector<int8_t>& mask, std::vector<double>& voltage);

// Field2D::load (src/Field2D.cpp:46-130): 'x y value' table
struct LoadedField {
    int nx = 0, nz = 0;
    double dx = 0, dz = 0, xmin = 0, zmin = 0;
    std::vector<double> v;
};
LoadedField load_field_table(const std::string& path, int ncols_value = 1, std::vector<double>* second = nullptr);

}  // namespace mag
