// The 3D Cartesian run (coord = CARTESIAN3D): ElMag3D + Species<CARTESIAN3D>
// of the reference (src/fields3d.hpp, src/fields3d.cpp:1-101,
// src/species3d.cpp:3-94, src/Field3D.hpp:40-163), on the GPU.
//
// The reference's 3D code is a prototype that does not build as shipped; this
// class follows its mathematics:
//  * geometry (Geometry::Geometry, fields3d.cpp:11-31): every node of the
//    box faces fixed at 0 V, and the one node of its "Quadrupole" electrode,
//    the centre (nx/2, ny/2, nz/2), fixed at the electrode's default 1 V;
//  * field: the 7-point Poisson problem (fields3d.cpp:35-101) with the grid
//    spacings, -lap(u) = rho / eps0 on the free nodes, rho = the particles'
//    trilinear charge (Field3D::accumulate) x macroparticle_factor / cell
//    volume; E = -grad u with the staggered differences of
//    Field3D::grad_component;
//  * particles: the leapfrog Boris step of Species<CARTESIAN3D>::advance with
//    constant B (the reference fixes B = 0), boundary FREE or PERIODIC,
//    t_grid::is_free over the cell's 8 corners, the charge deposit, and the
//    null-collision MCC of the 2D path (the scatter does not depend on the
//    dimension).
// A step is Pic::advance's: with selfconsistent = 1 a solve from the last
// deposits, then every species' push; without it the field of the electrode
// alone, solved at advance_init.
#pragma once

#include <string>
#include <vector>

#include "sim.hpp"

namespace mag {

class Sim3D {
public:
    Sim3D(const std::string& config, const std::string& species_conf, const SimOptions& opts);
    ~Sim3D();

    Param p;
    std::vector<SpeciesParams> species_prm;
    std::vector<InteractionParams> inters;
    std::vector<SpeciesState> sp;        // x, z, vx, vy, vz, id, counters, MCC data as in 2D
    std::vector<DevArray<uint32_t>> ys;  // the y coordinate of every species
    int nx = 0, ny = 0, nz = 0;
    double dx = 0, dy = 0, dz = 0, xmax = 0, ymax = 0, zmax = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    uint64_t seed = 1;
    int64_t launches = 0;
    double tol = 1e-12;
    int max_iter = 20000;
    std::vector<int8_t> mask;
    std::vector<double> voltage;
    SolveStatus last_solve{};

    void set_particles(int s, int64_t n, const double* x, const double* y, const double* z, const double* vx,
                       const double* vy, const double* vz);
    void get_particles(int s, int64_t cap, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                       uint32_t* id, int64_t* n_out);
    void advance_init();
    void advance(uint64_t nsteps);
    SolveStatus solve(const double* rho_host);  // rho_host: charge density [C/m^3] or null (the deposits)
    void get_field(int which, double* out);     // 0 u, 2 rho (charge density of the deposits), 3 mask
    void get_rho_fixed(int s, int64_t* out);
    Counters counters(int s);
    void energy(int s, double& sum_v2, unsigned long long& n);
    int sync();

private:
    bool own_stream = true;
    int sm_count = 0, solve_blocks = 0;
    DevArray<int8_t> d_mask;
    DevArray<uint8_t> d_cellfree;
    DevArray<double> d_volt, u, b, r, pv, qv, part, rho64, stage;
    DevArray<float> Exf, Eyf, Ezf;
    DevArray<unsigned> bar;
    DevArray<int> d_err;
    DevArray<SolveStatus> d_status;
    DevArray<InterDev> d_inter;
    DevArray<double> d_tables;
    DevArray<double> e_sum;
    DevArray<unsigned long long> e_cnt;

    void ensure_capacity(int s, int64_t need);
    void upload_slots(int s);
    Push3Args push_args(int s, bool init);
    CollideArgs collide_args(int s);
    void run_solve(bool from_rho64, bool clear_rho);
    void step();
};

}  // namespace mag
