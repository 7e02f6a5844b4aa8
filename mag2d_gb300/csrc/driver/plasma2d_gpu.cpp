// plasma2d_gpu: the reference's time-loop driver (src/test.cpp:18-97) on the
// GPU library, through the C ABI only.  Same command line:
//   plasma2d_gpu config=config.txt species_conf=species_conf.txt
//                initscript=initscript.txt output_dir=output [niter=N] [seed=S]
// Writes out.dat (iteration, wall seconds, live particles of every species)
// every t_print steps, the tracked particles' <species>_traj_<slot>.dat every
// 10 steps, <species>.dat (niter n_live mean_energy_eV t, the
// columns of BaseSpecies::print_status, src/particles.cpp:367-375) and, at
// the end, potential.dat in the x z value layout of Field2D::print
// (src/Field2D.cpp:30-44).  The reference's interactive y/n prompt before
// overwriting output_dir (src/output.cpp:12-32) is not reproduced.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <filesystem>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "mag2d_gpu.h"

static void die(const char* what)
{
    std::fprintf(stderr, "plasma2d_gpu: %s: %s\n", what, mag_last_error());
    std::exit(1);
}

int main(int argc, char** argv)
{
    std::map<std::string, std::string> cl = {{"config", "config.txt"},
                                             {"species_conf", "species_conf.txt"},
                                             {"initscript", "initscript.txt"},
                                             {"output_dir", "output"}};
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        const size_t eq = a.find('=');
        if (eq != std::string::npos) cl[a.substr(0, eq)] = a.substr(eq + 1);
    }
    double v;
    if (mag_config_param(cl["config"].c_str(), "niter", &v) != MAG_OK) die("config");
    unsigned long niter = cl.count("niter") ? std::stoul(cl["niter"]) : (unsigned long)v;
    mag_config_param(cl["config"].c_str(), "t_print", &v);
    const unsigned long t_print = (unsigned long)v;
    std::filesystem::create_directories(cl["output_dir"]);

    mag_opts o = {};
    o.seed = cl.count("seed") ? std::stoull(cl["seed"]) : 1;
    mag_sim* sim = nullptr;
    if (mag_create(cl["config"].c_str(), cl["species_conf"].c_str(), cl["initscript"].c_str(), &o, &sim) != MAG_OK)
        die("create");
    if (mag_advance_init(sim) != MAG_OK) die("advance_init");
    const int ns = mag_n_species(sim);
    std::vector<mag_species_info> info(ns);
    std::vector<std::ofstream> sp_out(ns);
    for (int s = 0; s < ns; ++s) {
        mag_species(sim, s, &info[s]);
        sp_out[s].open(cl["output_dir"] + "/" + info[s].name + ".dat");
    }
    std::ofstream out(cl["output_dir"] + "/out.dat");
    const auto t0 = std::chrono::steady_clock::now();
    // Pic::print_trace every 10 steps (src/test.cpp:66-69) when the initscript tracks particles
    bool trace = false;
    {
        std::ifstream ini(cl["initscript"]);
        std::string line;
        while (std::getline(ini, line)) trace = trace || line.find("add_tracked_particle") != std::string::npos;
    }
    unsigned long done = 0;
    while (done < niter) {
        unsigned long chunk = t_print ? std::min(t_print - done % t_print, niter - done) : niter - done;
        if (trace) chunk = std::min(chunk, 10 - done % 10);
        if (mag_advance(sim, chunk) != MAG_OK) die("advance");
        done += chunk;
        if (trace && done % 10 == 0 && mag_print_trace(sim, cl["output_dir"].c_str()) != MAG_OK) die("trace");
        if ((t_print && done % t_print == 0) || done == niter) {
            if (mag_sync(sim) != MAG_OK) die("advance");
            const double wall = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
            out << done << " " << wall;
            for (int s = 0; s < ns; ++s) {
                mag_diag_out d;
                if (mag_diag(sim, s, &d) != MAG_OK) die("diag");
                out << " " << d.n_live;
                sp_out[s] << d.niter << " " << d.n_live << " " << d.mean_energy_eV << " " << d.niter * info[s].dt
                          << "\n";
            }
            out << "\n";
        }
    }
    int nx, nz;
    double dx, dz, x0, z0;
    mag_grid(sim, &nx, &nz, &dx, &dz, &x0, &z0);
    std::vector<double> u((size_t)nx * nz);
    if (mag_get_field(sim, MAG_U, u.data()) != MAG_OK) die("field");
    std::ofstream pot(cl["output_dir"] + "/potential.dat");
    for (int i = 0; i < nx; ++i) {
        for (int j = 0; j < nz; ++j) pot << i * dx + x0 << "\t" << j * dz + z0 << "\t" << u[(size_t)i * nz + j] << "\n";
        pot << "\n";
    }
    mag_destroy(sim);
    return 0;
}
