// Host-side inputs: config.txt, species_conf, electrode geometry, field tables.
#include "host_config.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <limits>
#include <sstream>

namespace mag {

namespace {

std::string trim(const std::string& s)
{
    size_t a = s.find_first_not_of(" \t\r\n");
    if (a == std::string::npos) return "";
    size_t b = s.find_last_not_of(" \t\r\n");
    return s.substr(a, b - a + 1);
}

std::string read_file(const std::string& path)
{
    std::ifstream f(path);
    if (!f) throw Error(-6, "cannot open file " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

// double2int (src/util.cpp:22-28)
int double2int(double x, double eps = 1e-2)
{
    int res = (int)(x + 0.5);
    if (std::fabs(res - x) > eps) {
        char buf[96];
        std::snprintf(buf, sizeof buf, "double2int() %g is not integer", x);
        throw Error(-1, buf);
    }
    return res;
}

uint64_t to_u64(const std::string& s, const char* key)
{
    std::istringstream is(s);
    unsigned long long v;
    if (!(is >> v)) throw Error(-1, std::string("string2: error converting string ") + s + " (" + key + ")");
    return v;
}

}  // namespace

// ---------------------------------------------------------------------------
KeyValueConfig KeyValueConfig::from_file(const std::string& path)
{
    KeyValueConfig c;
    c.parse(read_file(path));
    return c;
}

KeyValueConfig KeyValueConfig::from_text(const std::string& text)
{
    KeyValueConfig c;
    c.parse(text);
    return c;
}

std::string KeyValueConfig::expand(const std::string& in, const std::string& section) const
{
    std::string s = in;
    for (int guard = 0; guard < 64; ++guard) {
        size_t open = s.rfind("${");
        if (open == std::string::npos) break;
        size_t close = s.find('}', open);
        if (close == std::string::npos) break;
        std::istringstream is(s.substr(open + 2, close - open - 2));
        std::vector<std::string> tok;
        for (std::string t; is >> t;) tok.push_back(t);
        std::string out;
        if (!tok.empty() && tok[0].size() == 1 && std::string("+-*/").find(tok[0][0]) != std::string::npos) {
            double acc = tok.size() > 1 ? std::atof(tok[1].c_str()) : 0.0;
            for (size_t i = 2; i < tok.size(); ++i) {
                double x = std::atof(tok[i].c_str());
                switch (tok[0][0]) {
                case '+': acc += x; break;
                case '-': acc -= x; break;
                case '*': acc *= x; break;
                default: acc /= x; break;
                }
            }
            char buf[64];
            std::snprintf(buf, sizeof buf, "%.17g", acc);
            out = buf;
        } else if (!tok.empty()) {
            auto it = vars_.find(section + tok[0]);
            if (it == vars_.end()) it = vars_.find(tok[0]);
            if (it != vars_.end()) out = it->second;
        }
        s = s.substr(0, open) + out + s.substr(close + 1);
    }
    return s;
}

void KeyValueConfig::parse(const std::string& text)
{
    std::istringstream f(text);
    std::string line, section;
    while (std::getline(f, line)) {
        size_t hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        line = trim(line);
        if (line.empty()) continue;
        if (line[0] == '[') {
            size_t close = line.find(']');
            std::string name = trim(line.substr(1, close == std::string::npos ? std::string::npos : close - 1));
            section = (name.empty() || name == "/") ? "" : name + "/";
            continue;
        }
        size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        std::string key = trim(line.substr(0, eq));
        std::string val = expand(trim(line.substr(eq + 1)), section);
        if (!val.empty() && val[0] == '\'') {
            size_t q = val.find('\'', 1);
            val = val.substr(1, q == std::string::npos ? std::string::npos : q - 1);
        } else {
            std::istringstream is(val);
            std::string first;
            is >> first;
            val = first;
        }
        vars_[section + key] = val;
    }
}

double KeyValueConfig::get(const std::string& key, double dflt) const
{
    auto it = vars_.find(key);
    if (it == vars_.end()) return dflt;
    double x;
    if (std::sscanf(it->second.c_str(), "%lf", &x) != 1) return dflt;
    return x;
}

std::string KeyValueConfig::get(const std::string& key, const char* dflt) const
{
    auto it = vars_.find(key);
    return it == vars_.end() ? std::string(dflt) : it->second;
}

// ---------------------------------------------------------------------------
// Param (src/param.cpp:12-143): same keys, defaults, validation and derived values
Param make_param(const KeyValueConfig& c)
{
    Param p;
    p.x_max = c.get("r_max", 1e-2);
    p.x_max = c.get("x_max", p.x_max);
    p.y_max = c.get("y_max", 1e-2);
    p.z_max = c.get("z_max", 1e-2);
    p.x_sampl = c.get("r_sampl", 100);
    p.x_sampl = c.get("x_sampl", p.x_sampl);
    p.y_sampl = c.get("y_sampl", 2);
    p.z_sampl = c.get("z_sampl", 100);
    p.n_particles_total = c.get("n_particles_total", 1e5);
    p.density_total = c.get("density_total", 1e11);
    p.pressure = c.get("pressure", 133.0);
    p.neutral_temperature = c.get("neutral_temperature", 300.0);
    p.probe_radius = c.get("probe_radius", 1e-4);
    p.probe_length = c.get("probe_length", 1e-2);
    p.u_probe = c.get("u_probe", -10.0);
    p.extern_field = c.get("extern_field", 100.0);
    p.electric_field_static_file = c.get("electric_field_static_file", "");
    p.electric_field_rf_file = c.get("electric_field_rf_file", "");
    p.electric_field_from_file = c.get("electric_field_from_file", 0) != 0;
    p.has_probe = c.get("has_probe", 0) != 0;
    p.magnetic_field_file = c.get("magnetic_field_file", "");
    p.magnetic_field_const = c.get("magnetic_field_const", 1) != 0;
    p.Br = c.get("Br", 0.0);
    p.Bz = c.get("Bz", 0.0);
    p.Bt = c.get("Bt", 0.0);
    p.niter = to_u64(c.get("niter", "100000"), "niter");
    p.dt_elon = c.get("dt_elon", 1e-11);
    p.selfconsistent = c.get("selfconsistent", 1) != 0;
    p.use_source = c.get("use_source", 0) != 0;
    p.u_smooth = c.get("u_smooth", 0) != 0;
    p.rf = c.get("rf", 1) != 0;
    p.rf_amplitude = c.get("rf_amplitude", 10.0);
    p.rf_U0 = c.get("rf_U0", 0.0);
    p.rf_omega = 2 * M_PI * c.get("rf_freq", 20e6);
    p.rf_omega = c.get("rf_omega", p.rf_omega);
    if (p.selfconsistent && p.rf) throw Error(-1, "Param: selfconsistent rf trap not implemented");
    if (p.selfconsistent && p.electric_field_from_file)
        throw Error(-1, "Param: selfconsistent with electric_field_from_file not implemented");
    p.t_print = to_u64(c.get("t_print", "0"), "t_print");
    p.t_print_dist = to_u64(c.get("t_print_dist", "0"), "t_print_dist");
    p.t_dist_sample = p.t_print > 10 ? p.t_print / 10 : 1;
    std::string te = c.get("t_equilib", "niter+1");
    p.t_equilib = te == "niter+1" ? p.niter + 1 : to_u64(te, "t_equilib");
    p.particle_reload = c.get("particle_reload", 0) != 0;
    p.particle_reload_dir = c.get("particle_reload_dir", ".");
    p.src_fact = c.get("src_fact", 20);
    p.neutral_density = p.pressure / (kKB * p.neutral_temperature);
    p.do_plot = c.get("do_plot", 1) != 0;

    std::string coord = c.get("coord", "CYLINDRICAL");
    if (coord == "CYLINDRICAL") p.coord = CYLINDRICAL;
    else if (coord == "CARTESIAN") p.coord = CARTESIAN;
    else if (coord == "CARTESIAN3D") p.coord = CARTESIAN3D;
    else throw Error(-1, "Param: unrecognized coord value " + coord);

    std::string bnd = c.get("boundary", "FREE");
    if (bnd == "FREE") p.boundary = BND_FREE;
    else if (bnd == "MIRROR") p.boundary = BND_MIRROR;
    else if (bnd == "PERIODIC") p.boundary = BND_PERIODIC;
    else throw Error(-1, "Param: unrecognized boundary value " + bnd);
    if (p.coord == CYLINDRICAL && p.boundary != BND_FREE)
        throw Error(-1, "Param: only FREE boundary condition in cylindrical coords is implemented");
    if (p.boundary == BND_MIRROR) throw Error(-1, "Param: MIRROR boundary condition not implemented");

    std::string mover = c.get("mover", "ADVANCE_BORIS");
    if (mover == "ADVANCE_BORIS") p.mover = ADVANCE_BORIS;
    else if (mover == "ADVANCE_MULTICOLL") p.mover = ADVANCE_MULTICOLL;
    else throw Error(-1, "Param: unrecognized mover value " + mover);

    static const std::map<std::string, Geometry> geos = {
        {"EMPTY", GEO_EMPTY}, {"PROBE", GEO_PROBE}, {"RF_22PT", GEO_RF_22PT}, {"RF_8PT", GEO_RF_8PT},
        {"RF_HAITRAP", GEO_RF_HAITRAP}, {"RF_QUAD", GEO_RF_QUAD}, {"MAC", GEO_MAC},
        {"PENNING", GEO_PENNING}, {"PENNING_SIMPLE", GEO_PENNING_SIMPLE}, {"TUBE", GEO_TUBE},
        {"PENNING_ENDCAP", GEO_PENNING_ENDCAP}};
    std::string g = c.get("geometry", "EMPTY");
    auto gi = geos.find(g);
    if (gi == geos.end()) throw Error(-1, "Param: unrecognized geometry value " + g);
    p.geometry = gi->second;

    p.dx = p.x_max / (p.x_sampl - 1);
    p.dz = p.z_max / (p.z_sampl - 1);
    p.idx = 1.0 / p.dx;
    p.idz = 1.0 / p.dz;
    p.macroparticle_factor = c.get("macroparticle_factor", 1e4);
    p.V = p.n_particles_total / p.density_total;
    p.dV = p.V / ((p.x_sampl - 1) * (p.z_sampl - 1));
    p.dy = p.dV / (p.dx * p.dz);
    if (p.coord == CYLINDRICAL) p.dy = 2 * M_PI / p.macroparticle_factor;
    p.idy = 1.0 / p.dy;

    p.u_endcap = c.get("u_endcap", -10.0);
    p.u_ring = c.get("u_ring", 0.0);
    int nseg = c.get("ring_segments", 0);
    for (int k = 0; k < nseg; ++k)
        p.u_segments.push_back(c.get("u_segment_" + std::to_string(k), p.u_ring));

    if (p.x_sampl < 2 || p.z_sampl < 2) throw Error(-1, "Param: x_sampl and z_sampl must be at least 2");
    if (p.coord == CARTESIAN3D) {
        // the 3D grid's own spacing and cell volume (the 2D formula above
        // derives dy from V; Field3D takes dy as a grid spacing)
        if (p.y_sampl < 2) throw Error(-1, "Param: y_sampl must be at least 2 in CARTESIAN3D");
        p.dy = p.y_max / (p.y_sampl - 1);
        p.idy = 1.0 / p.dy;
        p.dV = p.dx * p.dy * p.dz;
    }
    return p;
}

// ---------------------------------------------------------------------------
// config_parse (src/parser.cpp:25-147)
void parse_species_conf(const std::string& path, std::vector<SpeciesParams>& species,
                        std::vector<InteractionParams>& interactions)
{
    std::istringstream f(read_file(path));
    enum { INIT, DEFAULT, SPECIES, INTERACTION, CROSS_SECTION } state = INIT;
    std::string raw;
    auto num = [](const std::vector<std::string>& l, size_t k) {
        if (l.size() <= k) throw Error(-1, "config_parse: missing value after \"" + l[0] + "\"");
        std::istringstream is(l[k]);
        double v;
        if (!(is >> v)) throw Error(-1, "string2: error converting string " + l[k] + " to T");
        return v;
    };
    auto word = [](const std::vector<std::string>& l, size_t k) {
        if (l.size() <= k) throw Error(-1, "config_parse: missing value after \"" + l[0] + "\"");
        return l[k];
    };
    while (std::getline(f, raw)) {
        if (!raw.empty() && raw[0] == '#') continue;
        std::istringstream is(raw);
        std::vector<std::string> line;
        for (std::string t; is >> t;) line.push_back(t);
        if (line.empty()) continue;
        if (line[0] == "DEFAULT") { state = DEFAULT; continue; }
        if (line[0] == "SPECIES") { species.emplace_back(); state = SPECIES; continue; }
        if (line[0] == "INTERACTION") { interactions.emplace_back(); state = INTERACTION; continue; }
        if (state == INIT) throw Error(-1, "config_parse: unrecognized first config block");
        if (state == SPECIES) {
            SpeciesParams& s = species.back();
            const std::string& k = line[0];
            if (k == "NAME") s.name = word(line, 1);
            else if (k == "TYPE") {
                std::string t = word(line, 1);
                if (t == "NEUTRAL") s.type = NEUTRAL;
                else if (t == "ELECTRON") s.type = ELECTRON;
                else if (t == "ION") s.type = ION;
                else throw Error(-1, "config_parse: unrecognized first species type \"" + t + "\"");
            } else if (k == "MASS") s.mass = num(line, 1);
            else if (k == "CHARGE") s.charge = num(line, 1);
            else if (k == "DENSITY") s.density = num(line, 1);
            else if (k == "DT") s.dt = num(line, 1);
            else if (k == "TEMPERATURE") s.temperature = num(line, 1);
            else if (k == "EMAX") s.E_max = num(line, 1);
            else throw Error(-1, "config_parse: unrecognized species  parameter \"" + k + "\"");
        }
        if (state == INTERACTION) {
            InteractionParams& it = interactions.back();
            const std::string& k = line[0];
            if (k == "NAME") it.name = word(line, 1);
            else if (k == "TYPE") {
                std::string t = word(line, 1);
                if (t == "ELASTIC") it.type = ELASTIC;
                else if (t == "LANGEVIN") it.type = LANGEVIN;
                else if (t == "CX") it.type = CX;
                else if (t == "COULOMB") it.type = COULOMB;
                else if (t == "SUPERELASTIC") it.type = SUPERELASTIC;
                else throw Error(-1, "config_parse: unrecognized interaction type \"" + t + "\"");
            } else if (k == "DE") it.DE = num(line, 1);
            else if (k == "RATE") it.rate = num(line, 1);
            else if (k == "CUTOFF") it.cutoff = num(line, 1);
            else if (k == "PRIMARY") it.primary = word(line, 1);
            else if (k == "SECONDARY") it.secondary = word(line, 1);
            else if (k == "CROSS_SECTION") { state = CROSS_SECTION; continue; }
            else throw Error(-1, "config_parse: unrecognized species  parameter\"" + k + "\"");
        }
        if (state == CROSS_SECTION) {
            InteractionParams& it = interactions.back();
            if (line[0] == "END_CROSS_SECTION") state = INTERACTION;
            else {
                it.CS_energy.push_back(num(line, 0));
                it.CS_value.push_back(num(line, 1));
            }
        }
    }
}

// ---------------------------------------------------------------------------
double interaction_sigma_v(const InteractionParams& in, const std::vector<SpeciesParams>& sp, int prim, int sec,
                           double v)
{
    const double m1 = sp[prim].mass, m2 = sp[sec].mass;
    const double mu = m1 * m2 / (m1 + m2);
    const double EeV = 0.5 * mu * v * v / kQe;
    if (in.type == COULOMB) {  // Interaction::coulomb_sigma (src/particles.cpp:19-26)
        const double E = EeV * kQe;
        const SpeciesParams& P = sp[prim];
        const double lambda_D = std::sqrt(kEps0 * kKB * P.temperature / (P.density * P.charge * P.charge));
        const double Lambda = P.charge * sp[sec].charge / (4 * M_PI * kEps0 * E);
        return M_PI * Lambda * Lambda * std::log(lambda_D / Lambda) * v;
    }
    if (!in.CS_energy.empty()) {  // vec_interpolate (src/tabulate.cpp:124-140)
        const std::vector<double>& E = in.CS_energy;
        const std::vector<double>& S = in.CS_value;
        const int n = (int)E.size();
        double y;
        if (EeV >= E[n - 1]) y = S[n - 1];
        else if (EeV <= E[0]) y = S[0];
        else {
            int j1 = 0, j2 = n - 1;
            while (j2 - j1 > 1) {
                const int j3 = (j1 + j2) / 2;
                if (EeV < E[j3]) j2 = j3;
                else j1 = j3;
            }
            const double w = (EeV - E[j1]) / (E[j2] - E[j1]);
            y = S[j1] * (1 - w) + S[j2] * w;
        }
        return y * v;
    }
    return in.rate;
}

void species_rates(const std::vector<SpeciesParams>& sp, const std::vector<InteractionParams>& inters, int s,
                   std::vector<double>& rates, double& lifetime)
{
    const int ns = (int)sp.size();
    std::map<std::string, int> idx;
    for (int k = 0; k < ns; ++k) idx[sp[k].name] = k;
    const SpeciesParams& S = sp[s];
    const double E_max = S.E_max > 0. ? S.E_max : S.temperature * kKB / kQe * 10.0;
    const double vmax = std::sqrt(E_max * kQe / S.mass * 2.0);
    rates.assign(ns, 0.0);
    double rate = 0.0;
    for (int t = 0; t < ns; ++t) {
        std::vector<InteractionParams> list;
        for (const InteractionParams& in : inters) {
            auto pi = idx.find(in.primary), si = idx.find(in.secondary);
            if (pi == idx.end() || si == idx.end() || pi->second != s || si->second != t) continue;
            list.push_back(in);
            if (in.type == LANGEVIN) list.back().rate *= in.cutoff * in.cutoff;
        }
        double svmax = 0.0;
        if (!list.empty()) {
            const double dv = vmax / 1000;  // svmax_find with 1000 samples
            for (double v = 0; v < vmax; v += dv) {
                double sv = 0;
                for (const InteractionParams& in : list) sv += interaction_sigma_v(in, sp, s, t, v);
                if (std::isnan(sv)) continue;
                if (sv > svmax) svmax = sv;
            }
        }
        rates[t] = svmax * sp[t].density;
        rate += rates[t];
    }
    lifetime = rate > 0.0 ? 1.0 / rate : INFINITY;
}

// ---------------------------------------------------------------------------
// t_grid geometries (src/fields.cpp:374-868)
namespace {

struct Grid {
    int M, N;
    double dx, dz;
    std::vector<int8_t>& mask;
    std::vector<double>& volt;
    int8_t& m(int i, int j) { return mask[(size_t)i * N + j]; }
    double& v(int i, int j) { return volt[(size_t)i * N + j]; }

    // frame of the domain: which edges are electrodes
    void frame(bool axis_free, double vfn(const Grid&, int, int, const Param&), const Param& p)
    {
        for (int i = 0; i < M; i++)
            for (int j = 0; j < N; j++) {
                bool edge = (!axis_free && i == 0) || i == M - 1 || j == 0 || j == N - 1;
                if (edge) {
                    m(i, j) = FIXED;
                    v(i, j) = vfn(*this, i, j, p);
                } else
                    m(i, j) = FREE;
            }
    }
    void square_electrode(double rmin, double rmax, double zmin, double zmax, double vv, int8_t type = FIXED)
    {
        for (int i = 0; i < M; i++)
            for (int j = 0; j < N; j++) {
                double r = i * dx, z = j * dz;
                if (r > rmin && r < rmax && z > zmin && z < zmax) {
                    m(i, j) = type;
                    v(i, j) = vv;
                }
            }
    }
    void circle_electrode(double rc, double zc, double radius, double vv, int8_t type = FIXED)
    {
        double sq = radius * radius;
        for (int i = 0; i < M; i++)
            for (int j = 0; j < N; j++) {
                double r = i * dx - rc, z = j * dz - zc;
                if (r * r + z * z <= sq) {
                    m(i, j) = type;
                    v(i, j) = vv;
                }
            }
    }
    void mark_boundary()
    {
        for (int i = 2; i < M - 2; i++)
            for (int j = 2; j < N - 2; j++)
                if ((m(i - 1, j) == FIXED || m(i + 1, j) == FIXED || m(i, j - 1) == FIXED || m(i, j + 1) == FIXED) &&
                    m(i, j) != FIXED)
                    m(i, j) = BOUNDARY;
    }
    void multipole(int npoles, double r_pole, double r_rod)
    {
        double xc = 1e-2, yc = 1e-2;
        for (int i = 0; i < npoles; i++) {
            double x = xc + std::sin(2 * M_PI * (i + 1.0 / 32) / npoles) * r_pole;
            double y = yc + std::cos(2 * M_PI * (i + 1.0 / 32) / npoles) * r_pole;
            int sign = i % 2 == 0 ? -1 : 1;
            circle_electrode(x, y, r_rod, sign, FIXED_RF);
        }
    }
};

double v_zero(const Grid&, int, int, const Param&) { return 0.0; }
double v_ramp(const Grid& g, int, int j, const Param& p) { return -p.extern_field * g.dz * (j - g.N / 2); }

}  // namespace

void build_geometry(const Param& p, std::vector<int8_t>& mask, std::vector<double>& voltage)
{
    mask.assign((size_t)p.x_sampl * p.z_sampl, FREE);
    voltage.assign((size_t)p.x_sampl * p.z_sampl, 0.0);
    Grid g{p.x_sampl, p.z_sampl, p.dx, p.dz, mask, voltage};
    const int M = g.M, N = g.N;
    switch (p.geometry) {
    case GEO_PROBE:  // fields.cpp:437-473
        g.frame(false, v_ramp, p);
        g.circle_electrode((M - 1) * g.dx / 2, (N - 1) * g.dz / 2, p.probe_radius, p.u_probe, FIXED);
        g.mark_boundary();
        break;
    case GEO_RF_22PT:  // fields.cpp:475-519
        g.frame(false, v_zero, p);
        g.multipole(22, 0.75e-2, 0.05e-2);
        g.mark_boundary();
        break;
    case GEO_RF_8PT:  // fields.cpp:521-565
        g.frame(false, v_ramp, p);
        g.multipole(8, 0.3e-2 + 0.1e-2, 0.1e-2);
        g.mark_boundary();
        break;
    case GEO_RF_HAITRAP:  // fields.cpp:566-610
        g.frame(false, v_ramp, p);
        g.multipole(8, 0.3e-2 + 0.01e-2, 0.01e-2);
        g.mark_boundary();
        break;
    case GEO_TUBE: {  // fields.cpp:612-661
        g.frame(false, v_zero, p);
        double radius = p.probe_radius, rc = p.x_max / 2.0, zc = p.x_max / 2.0, sq = radius * radius;
        for (int i = 0; i < M; i++)
            for (int j = 0; j < N; j++) {
                double r = i * g.dx - rc, z = j * g.dz - zc;
                if (r * r + z * z >= sq) {
                    g.m(i, j) = FIXED;
                    g.v(i, j) = 0.0;
                }
            }
        g.mark_boundary();
    } break;
    case GEO_RF_QUAD:  // fields.cpp:663-699
        g.frame(false, v_zero, p);
        g.circle_electrode(5e-3, 1e-2, 2e-3, 1.0, FIXED_RF);
        g.circle_electrode(15e-3, 1e-2, 2e-3, 1.0, FIXED_RF);
        g.circle_electrode(1e-2, 5e-3, 2e-3, -1.0, FIXED_RF);
        g.circle_electrode(1e-2, 15e-3, 2e-3, -1.0, FIXED_RF);
        g.mark_boundary();
        break;
    case GEO_MAC: {  // fields.cpp:701-745
        g.frame(true, v_zero, p);
        g.square_electrode(5e-3, 4.5e-2, 1e-2, 1.5e-2, -.00);
        g.square_electrode(5e-3, 7e-3, 2e-2, 8e-2, 0.0);
        g.square_electrode(5e-3, 4.5e-2, 8.5e-2, 9e-2, -.00);
        double th = p.u_probe, ofs = 3e-2;
        g.square_electrode(3e-2, 3.3e-2, 11e-2 + ofs, 14e-2 + ofs, 0.8 * th);
        g.square_electrode(4.5e-2, 4.8e-2, 15e-2 + ofs, 25e-2 + ofs, th);
        g.square_electrode(3e-2, 3.3e-2, 26e-2 + ofs, 29e-2 + ofs, 1.0 * th);
        g.square_electrode(2.5e-2, 2.8e-2, 29e-2 + ofs, 30.5e-2 + ofs, 1.0 * th);
        g.square_electrode(15e-3, 4.5e-2, 35e-2, 35.3e-2, .0);
        g.square_electrode(0.0, 4.5e-2, 39.5e-2, 40e-2, 3e3);
        g.mark_boundary();
    } break;
    case GEO_PENNING:  // fields.cpp:747-788
        g.frame(true, v_zero, p);
        g.square_electrode(1.57e-2 / 2, 1.67e-2 / 2, 1e-3, 25e-3, -5);
        g.square_electrode(0, 1.46e-2 / 2, 15e-3, 16e-3, 10);
        g.square_electrode(0, 7e-3 / 2, 12e-3, 19e-3, 10);
        g.square_electrode(0, 1.9e-3, 1e-3, 12e-3, 10);
        g.square_electrode(4e-3, 7e-3, 52e-3, 53e-3, -5);
        g.square_electrode(2.5e-3, 7e-3, 46e-3, 47e-3, 0);
        g.mark_boundary();
        break;
    case GEO_PENNING_SIMPLE: {  // fields.cpp:790-833, trap_voltage = -1 (fields.hpp:173)
        g.frame(true, v_zero, p);
        double ri = 1e-2, ro = 1.1e-2;
        g.square_electrode(ri, ro, 0, 1e-2, -0.5);
        g.square_electrode(ri, ro, 1.1e-2, 2e-2, 0);
        g.square_electrode(ri, ro, 2.1e-2, 6e-2, -1.0);
        g.square_electrode(ri, ro, 6.1e-2, 7.5e-2, -10);
        g.mark_boundary();
    } break;
    case GEO_PENNING_ENDCAP: {
        // Orthogonal Penning trap in r-z: end caps at z = z_min and z = z_max,
        // ring wall at r = r_max, axis free.  With ring_segments = K the wall
        // is split into K equal z-segments biased by u_segment_0..K-1.
        const int K = (int)p.u_segments.size();
        for (int i = 0; i < M; i++)
            for (int j = 0; j < N; j++) {
                if (j == 0 || j == N - 1) {
                    g.m(i, j) = FIXED;
                    g.v(i, j) = p.u_endcap;
                } else if (i == M - 1 || (p.coord == CARTESIAN && i == 0)) {
                    g.m(i, j) = FIXED;
                    if (K > 0) {
                        int k = (int)((j * g.dz) / p.z_max * K);
                        if (k >= K) k = K - 1;
                        g.v(i, j) = p.u_segments[k];
                    } else
                        g.v(i, j) = p.u_ring;
                } else
                    g.m(i, j) = FREE;
            }
        g.mark_boundary();
    } break;
    case GEO_EMPTY:
    default:  // fields.cpp:417-435
        g.frame(false, v_ramp, p);
        break;
    }
}

// ---------------------------------------------------------------------------
// Field2D::load (src/Field2D.cpp:46-130) and Fields::load_magnetic_field
// (src/fields.cpp:870-959): ncols_value = 1 or 2 value columns.
LoadedField load_field_table(const std::string& path, int ncols_value, std::vector<double>* second)
{
    std::ifstream fr(path);
    if (fr.fail()) throw Error(-6, "Field2D::load(): failed opening file " + path);
    std::vector<double> xv, yv, fv, gv;
    std::string line;
    while (std::getline(fr, line)) {
        std::istringstream s(line);
        double a, b, c, d = 0;
        if (!(s >> a >> b >> c)) continue;
        if (ncols_value == 2 && !(s >> d)) continue;
        xv.push_back(a);
        yv.push_back(b);
        fv.push_back(c);
        gv.push_back(d);
    }
    if (xv.size() < 2) throw Error(-1, "Field2D::load(): too few samples in " + path);
    const double eps = ncols_value == 2 ? 1e-2 : 1e-1;
    LoadedField L;
    double xmin = xv[0], xmax = xv.back();
    size_t i = 1;
    while (i < xv.size() && xv[i] - xv[i - 1] == 0.0) i++;
    if (i == xv.size()) throw Error(-1, "Field2D::load(): x does not vary in " + path);
    double dx = xv[i] - xv[i - 1];
    if (dx < 0) { dx = -dx; xmin = xv.back(); xmax = xv[0]; }
    int nx = double2int((xmax - xmin) / dx + 1, eps);
    double ymin = yv[0], ymax = yv[xv.size() - 1];
    i = 1;
    while (i < yv.size() && yv[i] - yv[i - 1] == 0.0) i++;
    if (i == yv.size()) throw Error(-1, "Field2D::load(): y does not vary in " + path);
    double dy = yv[i] - yv[i - 1];
    if (dy < 0) { dy = -dy; ymin = yv.back(); ymax = yv[0]; }
    int ny = double2int((ymax - ymin) / dy + 1, eps);
    if ((size_t)nx * ny != xv.size()) throw Error(-1, "Fields::load_magnetic_field() wrong size of input vector");
    L.nx = nx; L.nz = ny; L.dx = dx; L.dz = dy; L.xmin = xmin; L.zmin = ymin;
    L.v.assign((size_t)nx * ny, std::numeric_limits<double>::quiet_NaN());
    if (second) second->assign((size_t)nx * ny, std::numeric_limits<double>::quiet_NaN());
    for (size_t k = 0; k < xv.size(); k++) {
        int xi = double2int((xv[k] - xmin) / dx, eps);
        int yi = double2int((yv[k] - ymin) / dy, eps);
        if (xi < 0 || xi >= nx || yi < 0 || yi >= ny) throw Error(-1, "Field2D::load(): sample outside grid");
        L.v[(size_t)xi * ny + yi] = fv[k];
        if (second) (*second)[(size_t)xi * ny + yi] = gv[k];
    }
    for (size_t k = 0; k < L.v.size(); k++)
        if (std::isnan(L.v[k]) || (second && std::isnan((*second)[k])))
            throw Error(-1, "Fields::load_magnetic_field() garbage loaded");
    return L;
}

}  // namespace mag
