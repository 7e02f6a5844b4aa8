// Host orchestration of the GPU time step: owns the device state of one
// simulation and issues the kernels of Pic::advance (src/pic.cpp:330-358).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

#include "device.hpp"
#include "host_config.hpp"

namespace mag {

void check_cuda(cudaError_t e, const char* what);
#define MAG_CK(call) ::mag::check_cuda((call), #call)

// Owning device allocation.
template <class T>
struct DevArray {
    T* p = nullptr;
    size_t n = 0;
    DevArray() = default;
    DevArray(const DevArray&) = delete;
    DevArray& operator=(const DevArray&) = delete;
    DevArray(DevArray&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
    DevArray& operator=(DevArray&& o) noexcept
    {
        if (this != &o) {
            release();
            p = o.p;
            n = o.n;
            o.p = nullptr;
            o.n = 0;
        }
        return *this;
    }
    ~DevArray() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void alloc(size_t count)
    {
        release();
        if (count == 0) return;
        MAG_CK(cudaMalloc((void**)&p, count * sizeof(T)));
        n = count;
    }
    void zero(cudaStream_t s)
    {
        if (n) MAG_CK(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
    void upload(const T* h, size_t count, cudaStream_t s)
    {
        if (count > n) alloc(count);
        if (count) MAG_CK(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void download(T* h, size_t count, cudaStream_t s) const
    {
        if (count) MAG_CK(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
};

struct SimOptions {
    int device = 0;
    uint64_t seed = 1;
    int sort_interval = 0;  // 0: default (20), < 0: never
    double poisson_tol = 1e-12;
    int poisson_max_iter = 200;
    int64_t capacity_hint = 0;
    int push_vec = 0;       // slots per thread of the particle kernel: 1, 2 or 4 (0: by particle count)
    int direct_solve = 0;   // Poisson by the precomputed inverse: 0 automatic (small grids), 1 forced, -1 never
    int max_fused_steps = 0;  // steps per fused particle launch where particles are independent (0: 64, 1: none)
    int multigrid_fp64 = 0;   // 1: every multigrid level in FP64 (one-block grids only)
    cudaStream_t stream = nullptr;  // work on this stream instead of one of its own (not destroyed)
};

class Batch;
class Adjoint;

struct SpeciesState {
    SpeciesParams prm;
    double v_max = 0, E_max = 0, lifetime = INFINITY, prob = 0;
    uint32_t threshold = 0;
    std::vector<double> rates;              // rates_by_species
    std::vector<std::vector<int>> by_target;  // interaction indices per target species
    // device particles (x, z fixed point, see device.hpp) and their sort double buffers
    DevArray<uint32_t> x, z, id, cand;
    DevArray<float4> cand_rec;
    DevArray<double> ttd;  // time to the next collision (ADVANCE_MULTICOLL), FP64
    DevArray<float> vx, vy, vz;
    DevArray<uint32_t> bx, bz, bid;
    DevArray<float> bvx, bvy, bvz;
    DevArray<MccSpecies> mcc;
    int64_t cap = 0, n_slots = 0;
    uint32_t next_id = 0;
    bool scrambled = false;            // slots filled in no cell order since the last sort (loaders, set_particles)
    DevArray<unsigned long long> rho;  // fixed-point charge grid
    DevArray<Counters> cnt;
    uint64_t niter = 0;                // steps advanced (Species::advance niter++, particles.hpp:347)
    uint64_t launches = 0;             // particle kernel launches (parity of the per-step counters)
    int inter_off = 0;                 // first entry of this species in the device interaction list
};

// Source box of one species (use_source, Species<CARTESIAN>::source2_particles)
struct SourceState {
    DevArray<double> x, z, rec;
    DevArray<float> vx, vy, vz;
    DevArray<int> count, offs;
    DevArray<long long> total;
    DevArray<unsigned long long> dropped;
    int64_t n = 0;
    int factor = 0;
    uint64_t injected = 0;  // copies appended to the species so far
};

struct SolverLevels {
    int nlev = 0;
    std::vector<int> nx, nz;
    std::vector<int> cmode;      // how level l is coarsened to level l + 1 (kCoarsen*)
    std::vector<DevArray<float>> e, r, t, coef, inv_diag;
    DevArray<float> coarse_inv;  // dense inverse of the coarsest level (column-major) or empty
    DevArray<float> coarse_inv_rows;  // multi-block grids: the same inverse row-major
    DevArray<double> st64;       // fine stencil rows (w, e, c)
    DevArray<double> rscale;     // right-hand-side scaling of rho per row
    DevArray<float> st32;
    double k2 = 1.0;
    // multi-block solves: tile phases of the levels above the single-block ones
    std::vector<int> ti, tj;     // tile interiors per level (empty: not yet chosen)
    std::vector<int> staged;     // Galerkin levels: 1 = tiles stage the operator, 0 = read from global memory
    size_t tile_smem = 0;        // dynamic shared memory of the launch (0: tile phases off)
    bool coarse_staged = false;  // block 0's levels fit the dynamic shared memory
    // the all-FP64 multigrid (SimOptions::multigrid_fp64): the same levels in FP64
    std::vector<DevArray<double>> e64, r64, t64, coef64, inv_diag64;
    DevArray<double> coarse_inv64;
};

void build_species(const std::vector<SpeciesParams>& species_prm, std::vector<InteractionParams>& inters,
                   size_t grid_nodes, cudaStream_t stream, std::vector<SpeciesState>& sp, DevArray<InterDev>& d_inter,
                   DevArray<double>& d_tables);

class Sim {
public:
    Sim(const std::string& config, const std::string& species_conf, const SimOptions& opts);
    ~Sim();

    void run_initscript(const std::string& path);
    void advance_init(bool deposit = true);  // deposit = false: solve from the species deposits as they are
    void advance(uint64_t nsteps);
    void advance_timed(uint64_t nsteps, double* ms4);
    int sync();  // returns first device error code (0 = none)
    // particle source (use_source): source5_refresh of every species with
    // particles, one step of a species' box, source5_save / source5_load
    std::vector<SourceState> src;
    void source_refresh(int factor);
    void source_step(int s);
    SourceArgs source_args(int s, bool init);
    void source_save(int s, const std::string& path);
    bool source_load(int s, const std::string& path);

    // accessors used by the C ABI
    std::string config_path;  // the config.txt the simulation was made from
    Param p;
    std::vector<SpeciesParams> species_prm;
    std::vector<InteractionParams> inters;
    std::vector<SpeciesState> sp;
    std::vector<int8_t> mask;
    std::vector<double> voltage;
    int nx = 0, nz = 0;
    double dx = 0, dz = 0, x0 = 0, z0 = 0, xmax = 0, zmax = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
    uint64_t seed = 1;
    int64_t launches = 0;
    double poisson_tol = 1e-12;
    int poisson_max_iter = 200;
    bool rho_override = false;
    SolveStatus last_solve{};
    int sort_interval = 20;
    int push_vec = 0;  // 1, 2 or 4 slots per thread of the particle kernel, 0: by particle count
    // slots per thread: 4 once a species has millions of slots (fewer chunk
    // flushes of the deposit tile and more loads in flight per thread,
    // measured faster on 1e8 electrons), else 2 (more threads for small runs)
    int push_vec_for(int64_t n) const { return push_vec ? push_vec : (n >= 4000000 ? 4 : 2); }
    int sm_count = 1;
    bool multicoll = false;  // mover ADVANCE_MULTICOLL
    int solve_blocks = 0;  // blocks of a cooperative solve (0: not yet chosen)
    int direct_mode = 0;   // SimOptions::direct_solve
    bool mg_fp64 = false;  // SimOptions::multigrid_fp64
    int max_fused = kMaxFusedSteps;  // SimOptions::max_fused_steps
    DevArray<double> stage64;  // host particle arrays on their way to the SoA state
    // the inverse of the Poisson operator for direct solves (built at the first self-consistent solve)
    DevArray<double> green, green_vac, green_b, green_part;
    DevArray<int> green_j;  // compacted right-hand side (node, value) and the per-tile counts
    // a step's solve computes only the nodes near charge (the particles'
    // cells); the rest of u follows on demand from the same right-hand side
    DevArray<int> green_rows;
    DevArray<uint8_t> green_charged;
    SolveArgs green_last{};
    bool u_partial = false;
    bool partial_rows = true;  // off: every direct solve computes every node
    // the multigrid solve of a step starts from 2 u_n - u_(n-1) (when extrapolate_u)
    DevArray<double> u_prev;
    DevArray<int> u_prev_valid;
    bool extrapolate_u = true;
    void ensure_full_u();
    // Fields::u_smooth after a step's solve (u_smooth = 1): u, then its faces
    DevArray<double> u_tmp;
    void smooth_u();
    // particles added by add_tracked_particle (TrackedParticle, particles.hpp:297-309)
    struct Tracked {
        int s;
        uint32_t id;
        int64_t slot;
        std::shared_ptr<std::ofstream> out;
    };
    std::vector<Tracked> tracked;
    // device status and diagnostics, read back through page-locked host memory
    DevArray<double> diag_dev;
    StatusHost* status_host = nullptr;  // written by the device (launch_gather_status)
    StatusHost* status_dev = nullptr;
    int gather_status(const double* energy);
    void set_voltages(const double* v, size_t n);
    DevArray<SolveStatus> green_status;
    int green_chunks_n = 0;
    GreenArgs green_args(bool vacuum) const;
    bool green_tried = false;
    bool green_ready() const { return green.p != nullptr; }
    void build_green();
    uint64_t steps_done = 0;
    bool sort_due = true;

    void get_field(int which, double* out);

    void get_faces(int component, float* out);  // Exf (0) or Ezf (1)
    void set_field(int which, const double* in);
    SolveStatus field_solve();
    void get_particles(int s, int64_t cap, double* x, double* z, double* vx, double* vy, double* vz, uint32_t* id,
                       int64_t* n_out);
    void set_particles(int s, int64_t n, const double* x, const double* z, const double* vx, const double* vy,
                       const double* vz);
    void deposit_all();
    void get_rho_fixed(int s, int64_t* out);
    void set_rho_fixed(int s, const int64_t* in);
    // sampled distributions (BaseSpecies::dist_sample / dist_reset, Pic::dist_sample)
    void dist_reset();
    void dist_sample();
    int dist_samples() const { return nsampl; }
    // Histogram of species s: bin centres, print values (data / norm), stats (n_val, sum, n_val_tot, sum_tot)
    void energy_dist(int s, std::vector<double>& pos, std::vector<double>& val, double stats[4]);
    void average(int which, double* out);  // MAG_U: uAvg / nsampl; MAG_SPECIES_RHO + s: rhoAverage / nsampl
    void print_distribution(const std::string& dir);
    void print_field(const std::string& path);
    void print_trace(const std::string& dir);  // Pic::print_trace
    void save_species(int s, const std::string& path);  // BaseSpecies::save
    void load_species(int s, const std::string& path);  // BaseSpecies::load
    Counters counters(int s);
    void energy(int s, double& sum_v2, unsigned long long& n);
    int diag(int s, double& sum_v2, unsigned long long& n, Counters& c);
    uint64_t niter(int s);
    int solver_levels() const { return lv.nlev; }
    int solve_phase_times(double* out, int cap);

private:
    friend class Batch;
    friend class Adjoint;
    bool own_stream = true;
    int emode = 1;
    bool check_mask = true;
    DevArray<int8_t> d_mask;
    struct DistState {
        DevArray<unsigned long long> bins;  // energy_dist counts (200 bins over [0, E_max])
        DevArray<double> stats;             // n_val, sum, n_val_tot, sum_tot
        DevArray<double> rho_sum;           // sum of sampled rho [C per macro particle]
    };
    std::vector<DistState> dist;
    DevArray<double> u_sum;
    DevArray<unsigned long long> rho_scratch;
    int nsampl = 0;
    static constexpr int kEnergyBins = 200;  // energy_dist(200, 0, E_max), src/particles.hpp:169
    DevArray<uint8_t> d_cellfree;
    DevArray<double> d_volt, u64, urf64, b64, rho64, red;
    DevArray<float> Exf, Ezf, Exf_rf, Ezf_rf, d_Br, d_Bz;
    DevArray<float2> Exf2, Ezf2;
    DevArray<uint32_t> sort_count, sort_offset, sort_blocksum;
    int bnx = 0, bnz = 0;
    double b_x0 = 0, b_z0 = 0, b_dx = 1, b_dz = 1;
    DevArray<SolveStatus> d_status;
    DevArray<GridBarrier> d_bar;
    DevArray<int> d_err;
    DevArray<InterDev> d_inter;
    DevArray<double> d_tables;
    SolverLevels lv;
    bool solver_ready = false;
    DevArray<double> d_prof;  // phase times of the last multigrid solve [ns] once timing is on
    bool prof_on = false;

    void setup_fields();
    void setup_species();
    void setup_solver();
    void validate_operator() const;
    SolveStatus solve(bool rf_solve, int rho_src, bool clear_rho, bool wait);
    SolveArgs solve_args(bool rf_solve, int rho_src, bool clear_rho);
    void run_solve(SolveArgs a);  // launch (one block, or cooperative for large grids)
    void ensure_capacity(int s, int64_t need);
    void add_loaded(int s, int64_t n, int kind, double cx, double cz, double radius, double zlo, double zhi);
    void add_single(int s, double x, double z, double vx, double vy, double vz);
    PushArgs push_args(int s, bool init);
    CollideArgs collide_args(int s);
    void step(double* ms = nullptr);
    // steps the next fused launch can take (1: step by step), and the launch
    int fused_steps(uint64_t left) const;
    void fused_block(int nsteps, double* ms = nullptr);
    float rf_factor(uint64_t niter, double dt) const;
    void sort_species(int s);
    bool cell_order_broken(const double* x, const double* z, int64_t n) const;
    void refresh_rf_pairs();
    void upload_slots(int s);
    void init_ttd(int s, int64_t first, int64_t n);
    int coll_mode(int s) const;
    bool any_target_slots(int s) const;
};

}  // namespace mag
