// Host orchestration of the GPU PIC-MCC step.
#include "sim.hpp"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <map>
#include <mutex>
#include <sstream>
#include <string>

#include "kernels.hpp"
#include "multigrid_host.hpp"
#include "particle_io.hpp"

namespace mag {

void check_cuda(cudaError_t e, const char* what)
{
    if (e != cudaSuccess) throw Error(-2, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {

constexpr double kPi = 3.14159265358979323846;

bool fixed_node(int8_t m) { return m == FIXED || m == FIXED_RF; }

std::vector<std::string> tokens(const std::string& line)
{
    std::istringstream is(line);
    std::vector<std::string> t;
    for (std::string s; is >> s;) t.push_back(s);
    return t;
}

double to_num(const std::string& s)
{
    std::istringstream is(s);
    double v;
    if (!(is >> v)) throw Error(-1, "string2: error converting string " + s + " to T");
    return v;
}

int to_int(const std::string& s)
{
    std::istringstream is(s);
    int v;
    if (!(is >> v)) throw Error(-1, "string2: error converting string " + s + " to T");
    return v;
}

}  // namespace

// ---------------------------------------------------------------------------
Sim::Sim(const std::string& config, const std::string& species_conf, const SimOptions& opts)
{
    device = opts.device;
    seed = opts.seed;
    poisson_tol = opts.poisson_tol > 0 ? opts.poisson_tol : 1e-12;
    poisson_max_iter = opts.poisson_max_iter > 0 ? opts.poisson_max_iter : 200;
    sort_interval = opts.sort_interval == 0 ? 20 : opts.sort_interval;
    push_vec = opts.push_vec == 1 || opts.push_vec == 2 || opts.push_vec == 4 ? opts.push_vec : 0;
    direct_mode = opts.direct_solve;
    mg_fp64 = opts.multigrid_fp64 != 0;
    max_fused = opts.max_fused_steps <= 0 ? kMaxFusedSteps : std::min(opts.max_fused_steps, kMaxFusedSteps);
    if (cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sm_count < 1)
        sm_count = 1;
    config_path = config;
    p = make_param(KeyValueConfig::from_file(config));
    if (p.coord == CARTESIAN3D) throw Error(-1, "coord = CARTESIAN3D: use the 3D handle (mag3d_create)");
    multicoll = p.mover == ADVANCE_MULTICOLL;
    if (p.u_smooth) {
        // the smoothing reads every node, and the extrapolated start of the
        // next solve would extrapolate smoothed potentials
        partial_rows = false;
        extrapolate_u = false;
    }
    if (multicoll) {  // the reference's own conditions (src/particles.cpp:812-823)
        if (p.coord != CARTESIAN) throw Error(-1, "Species<CYLINDRICAL>: advance method not implemented");
        if (!p.magnetic_field_const || p.Br != 0.0 || p.Bt != 0.0 || p.Bz != 0.0)
            throw Error(-1, "Species<CARTESIAN>::advance_multicoll() implemented for zero B only");
        if (p.selfconsistent || p.geometry != GEO_EMPTY)
            throw Error(-1, "Species<CARTESIAN>::advance_multicoll() implemented for const extern field only:\n"
                            "\tset selfconsistent=0 and geometry=EMPTY");
    }
    if (p.use_source && p.coord != CARTESIAN)  // declared but never defined in the reference (particles.hpp:311)
        throw Error(-1, "use_source: Species<CYLINDRICAL>::source is not defined in the reference");
    if (p.use_source && multicoll)
        throw Error(-1, "use_source: the source box with ADVANCE_MULTICOLL is not provided by this library");
    parse_species_conf(species_conf, species_prm, inters);
    if (species_prm.empty()) throw Error(-1, "species_conf defines no species");
    if ((int)species_prm.size() > kMaxSpecies) throw Error(-1, "too many species");
    if ((int)inters.size() > kMaxInteractions) throw Error(-1, "too many interactions");
    build_geometry(p, mask, voltage);
    MAG_CK(cudaSetDevice(device));
    if (opts.stream) {
        stream = opts.stream;
        own_stream = false;
    } else {
        MAG_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    }
    d_err.alloc(1);
    d_err.zero(stream);
    d_status.alloc(1);
    d_status.zero(stream);
    d_bar.alloc(1);
    d_bar.zero(stream);
    red.alloc(8);
    red.zero(stream);
    setup_fields();
    setup_species();
    if (opts.capacity_hint > 0)
        for (size_t s = 0; s < sp.size(); ++s) ensure_capacity((int)s, opts.capacity_hint);
    src.resize(sp.size());
    if (p.particle_reload)  // Pic constructor (src/pic.cpp:138-146): every species from particle_reload_dir
        for (size_t s = 0; s < sp.size(); ++s) {
            load_species((int)s, p.particle_reload_dir + "/particles_" + species_prm[s].name + ".dat");
            if (p.use_source) source_load((int)s, p.particle_reload_dir + "/particles_source_" + species_prm[s].name + ".dat");
        }
    MAG_CK(cudaStreamSynchronize(stream));
    int e = sync();
    if (e != 0) throw Error(e, "initial field solve failed (device status " + std::to_string(e) + ")");
}

Sim::~Sim()
{
    if (stream) {
        cudaSetDevice(device);
        cudaStreamSynchronize(stream);
        sp.clear();
        lv = SolverLevels{};
        if (status_host) cudaFreeHost(status_host);
        if (own_stream) cudaStreamDestroy(stream);
    }
}

int Sim::sync() { return gather_status(nullptr); }

// Waits for the stream; one kernel gathers the error flag, the solve status,
// the counters and optionally the energy sums into page-locked host memory
int Sim::gather_status(const double* energy)
{
    if (!status_host) {
        MAG_CK(cudaHostAlloc((void**)&status_host, sizeof(StatusHost), cudaHostAllocMapped));
        MAG_CK(cudaHostGetDevicePointer((void**)&status_dev, status_host, 0));
    }
    StatusSources src{};
    src.err = d_err.p;
    src.st = d_status.p;
    src.nsp = (int)sp.size();
    src.energy = energy;
    for (size_t s = 0; s < sp.size(); ++s) src.cnt[s] = sp[s].cnt.p;
    launches += launch_gather_status(src, status_dev, stream);
    MAG_CK(cudaStreamSynchronize(stream));
    int err = status_host->err;
    last_solve = status_host->st;
    for (size_t k = 0; k < sp.size(); ++k) {
        SpeciesState& s = sp[k];
        if (!s.cnt.p) continue;
        const Counters& c = status_host->c[k];
        if (c.error && !err) err = c.error;
        if (s.n_slots > 0 && (int64_t)c.slots < s.n_slots) s.n_slots = (int64_t)c.slots;
    }
    if (err) {
        int zero = 0;
        MAG_CK(cudaMemcpy(d_err.p, &zero, sizeof(int), cudaMemcpyHostToDevice));
    }
    return err;
}

// Fields: geometry, loaded or solved u and uRF, magnetic tables (pic.cpp:127-189)
void Sim::setup_fields()
{
    if (p.electric_field_from_file) {
        LoadedField u = load_field_table(p.electric_field_static_file);
        nx = u.nx;
        nz = u.nz;
        dx = u.dx;
        dz = u.dz;
        x0 = u.xmin;
        z0 = u.zmin;
        xmax = x0 + (nx - 1) * dx;
        zmax = z0 + (nz - 1) * dz;
        u64.upload(u.v.data(), u.v.size(), stream);
        urf64.alloc(u.v.size());
        urf64.zero(stream);
        if (p.rf) {
            LoadedField r = load_field_table(p.electric_field_rf_file);
            if (r.nx != nx || r.nz != nz || r.dx != dx || r.dz != dz || r.xmin != x0 || r.zmin != z0)
                throw Error(-1, "electric_field_rf_file grid differs from electric_field_static_file grid");
            urf64.upload(r.v.data(), r.v.size(), stream);
        }
        check_mask = false;  // advance_boundary skips is_free in this mode (particles.hpp:395)
    } else {
        nx = p.x_sampl;
        nz = p.z_sampl;
        dx = p.dx;
        dz = p.dz;
        x0 = 0;
        z0 = 0;
        xmax = p.x_max;
        zmax = p.z_max;
        u64.alloc((size_t)nx * nz);
        u64.zero(stream);
        urf64.alloc((size_t)nx * nz);
        urf64.zero(stream);
        check_mask = true;
    }
    if (nx - 1 > kMaxCellsPerAxis || nz - 1 > kMaxCellsPerAxis || nx < 2 || nz < 2)
        throw Error(-1, "field grid must have 2..4096 nodes per axis (fixed-point particle positions)");
    const size_t nn = (size_t)nx * nz;
    b64.alloc(std::max(nn, mask.size()));
    rho64.alloc(nn);
    rho64.zero(stream);
    Exf.alloc((size_t)(nx + 1) * nz);
    Ezf.alloc((size_t)nx * (nz + 1));
    Exf_rf.alloc((size_t)(nx + 1) * nz);
    Ezf_rf.alloc((size_t)nx * (nz + 1));
    Exf2.alloc((size_t)(nx + 1) * nz);
    Ezf2.alloc((size_t)nx * (nz + 1));
    sort_count.alloc((size_t)(nx - 1) * (nz - 1));
    sort_count.zero(stream);
    sort_offset.alloc((size_t)(nx - 1) * (nz - 1) + 1);
    sort_blocksum.alloc(((size_t)(nx - 1) * (nz - 1) + 1023) / 1024 + 1);
    d_mask.upload(mask.data(), mask.size(), stream);
    d_volt.upload(voltage.data(), voltage.size(), stream);
    {  // t_grid::is_free per cell (src/fields.hpp:94-101): one of the four corner nodes is FREE
        std::vector<uint8_t> cf((size_t)(nx - 1) * (nz - 1), 1);
        if (check_mask)
            for (int i = 0; i + 1 < nx; ++i)
                for (int j = 0; j + 1 < nz; ++j) {
                    const int8_t* m = mask.data() + (size_t)i * nz + j;
                    cf[(size_t)i * (nz - 1) + j] = (m[0] == 2 || m[nz] == 2 || m[1] == 2 || m[nz + 1] == 2) ? 1 : 0;
                }
        d_cellfree.upload(cf.data(), cf.size(), stream);
    }
    if (p.geometry == GEO_EMPTY && !p.selfconsistent) emode = 0;
    else emode = p.rf ? 2 : 1;
    if (!p.magnetic_field_const) {
        std::vector<double> bz;
        LoadedField br = load_field_table(p.magnetic_field_file, 2, &bz);
        std::vector<float> f1(br.v.begin(), br.v.end()), f2(bz.begin(), bz.end());
        d_Br.upload(f1.data(), f1.size(), stream);
        d_Bz.upload(f2.data(), f2.size(), stream);
        bnx = br.nx;
        bnz = br.nz;
        b_x0 = br.xmin;
        b_z0 = br.zmin;
        b_dx = br.dx;
        b_dz = br.dz;
    }
    if (p.electric_field_from_file) {
        launches += launch_faces(u64.p, nx, nz, dx, dz, Exf.p, Ezf.p, stream);
        launches += launch_faces(urf64.p, nx, nz, dx, dz, Exf_rf.p, Ezf_rf.p, stream);
    } else {
        // Pic constructor: boundary_solve_rf always, boundary_solve when not self-consistent
        setup_solver();
        solve(true, 0, false, false);
        if (!p.selfconsistent) solve(false, 0, false, false);
        else launches += launch_faces(u64.p, nx, nz, dx, dz, Exf.p, Ezf.p, stream);
    }
    refresh_rf_pairs();
}

// (u, uRF) face pairs for the RF gather
void Sim::refresh_rf_pairs()
{
    if (emode != 2) return;
    launches += launch_interleave(Exf.p, Exf_rf.p, Exf2.p, (long long)(nx + 1) * nz, stream);
    launches += launch_interleave(Ezf.p, Ezf_rf.p, Ezf2.p, (long long)nx * (nz + 1), stream);
}

void Sim::upload_slots(int s)
{
    const unsigned long long v = (unsigned long long)sp[s].n_slots;
    MAG_CK(cudaMemcpyAsync(&sp[s].cnt.p->slots, &v, sizeof v, cudaMemcpyHostToDevice, stream));
    MAG_CK(cudaStreamSynchronize(stream));
}

void Sim::validate_operator() const
{
    for (int i = 0; i < p.x_sampl; ++i)
        for (int j = 0; j < p.z_sampl; ++j) {
            if (fixed_node(mask[(size_t)i * p.z_sampl + j])) continue;
            const bool axis_ok = p.coord == CYLINDRICAL && i == 0;
            if ((i == 0 && !axis_ok) || i == p.x_sampl - 1 || j == 0 || j == p.z_sampl - 1)
                throw Error(-1, "geometry leaves a free node on the domain edge at (" + std::to_string(i) + "," +
                                    std::to_string(j) + "); the reference operator (fields.cpp:136-259) is undefined there");
        }
}

void Sim::setup_solver()
{
    if (solver_ready) return;
    validate_operator();
    const int coord = p.coord == CYLINDRICAL ? 1 : 0;
    std::vector<int> lnx, lnz, lmode;
    // couplings of the fine operator: r ones ~ 1/dx^2, z ones 1/dz^2 (cylindrical); unit in Cartesian runs
    // grids solved by all blocks stop at a larger coarsest level, which every block helps to solve
    const bool multi_block = (long long)nx * nz > kSingleBlockNodes;
    multigrid_levels(nx, nz, coord == 1 ? (dz * dz) / (dx * dx) : 1.0, kMaxLevels, lnx, lnz, lmode,
                     multi_block ? kDenseCoarseGridMax : kDenseCoarseMax);
    lv.nlev = (int)lnx.size();
    lv.nx = lnx;
    lv.nz = lnz;
    lv.cmode.assign(lv.nlev, kCoarsenFull);
    for (int l = 0; l + 1 < lv.nlev; ++l) lv.cmode[l] = lmode[l + 1];
    lv.e.resize(lv.nlev);
    lv.r.resize(lv.nlev);
    lv.t.resize(lv.nlev);
    lv.coef.resize(lv.nlev);
    lv.inv_diag.resize(lv.nlev);
    if (mg_fp64) {
        if ((long long)nx * nz > kSingleBlockNodes)
            throw Error(-1, "multigrid_fp64: the FP64 multigrid runs on one block, grids up to " +
                                        std::to_string(kSingleBlockNodes) + " nodes");
        for (auto* v : {&lv.e64, &lv.r64, &lv.t64, &lv.coef64, &lv.inv_diag64}) v->resize(lv.nlev);
    }
    std::vector<double> A, Ac;
    fine_operator(coord, nx, nz, dx, dz, mask, A);
    std::vector<char> fixed_f(mask.size());
    for (size_t k = 0; k < mask.size(); ++k) fixed_f[k] = fixed_node(mask[k]);
    for (int l = 0; l < lv.nlev; ++l) {
        const size_t n = (size_t)lnx[l] * lnz[l];
        lv.e[l].alloc(n);
        lv.r[l].alloc(n);
        lv.t[l].alloc(n);
        lv.e[l].zero(stream);
        if (mg_fp64) {
            lv.e64[l].alloc(n);
            lv.r64[l].alloc(n);
            lv.t64[l].alloc(n);
            lv.e64[l].zero(stream);
        }
        if (l == 0) continue;
        int cx, cz;
        galerkin(lnx[l - 1], lnz[l - 1], A, fixed_f, lmode[l], cx, cz, Ac);
        std::vector<float> cf(Ac.begin(), Ac.end()), idg(n);
        for (size_t k = 0; k < n; ++k) idg[k] = (float)(1.0 / Ac[4 * n + k]);
        lv.coef[l].upload(cf.data(), cf.size(), stream);
        lv.inv_diag[l].upload(idg.data(), idg.size(), stream);
        if (mg_fp64) {
            std::vector<double> idg64(n);
            for (size_t k = 0; k < n; ++k) idg64[k] = 1.0 / Ac[4 * n + k];
            lv.coef64[l].upload(Ac.data(), Ac.size(), stream);
            lv.inv_diag64[l].upload(idg64.data(), idg64.size(), stream);
        }
        MAG_CK(cudaStreamSynchronize(stream));
        A.swap(Ac);
        fixed_f.assign(n, 0);
    }
    // coarsest level solved exactly when small (A holds its operator now); the
    // inverse depends only on the operator, so instances that share grid and
    // geometry (batched sweeps) compute it once per process
    lv.coarse_inv.release();
    lv.coarse_inv_rows.release();
    if (lv.nlev > 1 && (long long)lnx.back() * lnz.back() <= (multi_block ? kDenseCoarseGridMax : kDenseCoarseMax)) {
        static std::mutex mu;
        static std::map<std::string, std::vector<float>> cache;
        std::string key((const char*)A.data(), A.size() * sizeof(double));
        key += std::to_string(lnx.back()) + "x" + std::to_string(lnz.back());
        std::vector<float> inv;
        bool found = false;
        {
            std::lock_guard<std::mutex> lock(mu);
            auto it = cache.find(key);
            if (it != cache.end()) {
                inv = it->second;
                found = true;
            }
        }
        if (!found && dense_inverse(lnx.back(), lnz.back(), A, inv)) {
            std::lock_guard<std::mutex> lock(mu);
            if (cache.size() > 64) cache.clear();
            cache[key] = inv;
        }
        if (!inv.empty()) lv.coarse_inv.upload(inv.data(), inv.size(), stream);
        if (!inv.empty() && multi_block) {
            const size_t n = (size_t)lnx.back() * lnz.back();
            std::vector<float> rows(n * n);
            for (size_t r = 0; r < n; ++r)
                for (size_t c = 0; c < n; ++c) rows[r * n + c] = inv[c * n + r];
            lv.coarse_inv_rows.upload(rows.data(), rows.size(), stream);
            MAG_CK(cudaStreamSynchronize(stream));
        }
        std::vector<double> inv64;
        if (mg_fp64 && dense_inverse64(lnx.back(), lnz.back(), A, inv64))
            lv.coarse_inv64.upload(inv64.data(), inv64.size(), stream);
    }
    std::vector<double> st;
    fine_stencil_table(coord, nx, dx, dz, st, lv.k2);
    std::vector<float> st32(st.begin(), st.end());
    lv.st64.upload(st.data(), st.size(), stream);
    lv.st32.upload(st32.data(), st32.size(), stream);
    // the right-hand-side scaling of rho per grid row (fields.cpp:283-300), the
    // same expression in the same order as the device would evaluate per node
    std::vector<double> rs(nx);
    for (int i = 0; i < nx; ++i)
        rs[i] = p.coord == CYLINDRICAL
                    ? (i > 0 ? -1.0 / kEps0 / (kPi * dx * dx * 2.0 * i * dz) * p.macroparticle_factor
                             : -1.0 / kEps0 / (kPi * dx * dx * 0.25 * dz) * p.macroparticle_factor)
                    : -(dx * dx) / kEps0 / p.dV;
    lv.rscale.upload(rs.data(), rs.size(), stream);
    MAG_CK(cudaStreamSynchronize(stream));
    solver_ready = true;
}

SolveStatus Sim::solve(bool rf_solve, int rho_src, bool clear_rho, bool wait)
{
    run_solve(solve_args(rf_solve, rho_src, clear_rho));
    SolveStatus st{};
    if (wait) {
        MAG_CK(cudaStreamSynchronize(stream));
        MAG_CK(cudaMemcpy(&st, d_status.p, sizeof st, cudaMemcpyDeviceToHost));
        last_solve = st;
    }
    return st;
}

// Inverse of the Poisson operator for the direct solve: column j is the
// solution for a unit right-hand side at node j with zero Dirichlet values,
// computed by batched single-block multigrid solves (chunks of columns at a
// time).  Only for grids of at most kGreenMaxNodes whose inverse fits in a
// quarter of the free device memory.
void Sim::build_green()
{
    green_tried = true;
    const long long nn = (long long)nx * nz;
    if (nn > kGreenMaxNodes && direct_mode != 1) return;
    if (nn > kSingleBlockNodes) return;  // columns are single-block solves
    size_t fr = 0, tot = 0;
    MAG_CK(cudaMemGetInfo(&fr, &tot));
    const size_t gbytes = (size_t)nn * nn * sizeof(double);
    if (gbytes > fr / 4) return;
    setup_solver();
    green.alloc((size_t)nn * nn);
    green.zero(stream);
    DevArray<double> zeros, bscr;
    zeros.alloc(nn);
    zeros.zero(stream);
    const int C = (int)std::max<long long>(1, std::min<long long>(1024, (256LL << 20) / (nn * 40)));
    bscr.alloc((size_t)C * nn);
    std::vector<DevArray<float>> e(lv.nlev), r(lv.nlev), t(lv.nlev);
    for (int l = 0; l < lv.nlev; ++l) {
        const size_t n = (size_t)lv.nx[l] * lv.nz[l] * C;
        e[l].alloc(n);
        r[l].alloc(n);
        t[l].alloc(n);
    }
    DevArray<SolveStatus> st;
    st.alloc(C);
    DevArray<SolveArgs> d_args;
    d_args.alloc(C);
    std::vector<SolveArgs> args;
    std::vector<long long> cols;
    for (long long k = 0; k < nn; ++k)
        if (!(mask[k] == 0 || mask[k] == 1)) cols.push_back(k);
    SolveArgs base = solve_args(false, 3, false);
    base.voltage = zeros.p;
    base.Exf = nullptr;
    base.Ezf = nullptr;
    base.tol = std::min(poisson_tol, 1e-12);
    for (size_t c0 = 0; c0 < cols.size(); c0 += C) {
        const int m = (int)std::min<size_t>(C, cols.size() - c0);
        args.assign(m, base);
        for (int c = 0; c < m; ++c) {
            SolveArgs& a = args[c];
            a.unit_node = cols[c0 + c];
            a.u = green.p + cols[c0 + c] * nn;
            a.b = bscr.p + (size_t)c * nn;
            for (int l = 0; l < lv.nlev; ++l) {
                const size_t n = (size_t)lv.nx[l] * lv.nz[l];
                a.lev[l].e = e[l].p + c * n;
                a.lev[l].r = r[l].p + c * n;
                a.lev[l].t = t[l].p + c * n;
            }
            a.status = st.p + c;
        }
        d_args.upload(args.data(), m, stream);
        launches += launch_solve_batch(d_args.p, m, 512, stream);
        std::vector<SolveStatus> hs(m);
        MAG_CK(cudaMemcpyAsync(hs.data(), st.p, m * sizeof(SolveStatus), cudaMemcpyDeviceToHost, stream));
        MAG_CK(cudaStreamSynchronize(stream));  // args and scratch are reused by the next chunk
        for (int c = 0; c < m; ++c)
            if (!hs[c].converged) {
                green.release();  // a column that did not converge: keep solving by multigrid
                return;
            }
    }
    MAG_CK(cudaGetLastError());
    green_chunks_n = green_chunks(nn, sm_count);
    green_b.alloc(nn);
    green_j.alloc(nn + (nn + 1023) / 1024);
    const long long ntiles = (nn + 1023) / 1024;
    green_rows.alloc((size_t)(ntiles * 1024 + ntiles));
    green_charged.alloc(nn);
    green_part.alloc((size_t)green_chunks_n * nn);
    green_status.alloc(1);
    // the potential of the electrodes alone
    green_vac.alloc(nn);
    SolveArgs v = solve_args(false, 0, false);
    v.u = green_vac.p;
    v.Exf = nullptr;
    v.Ezf = nullptr;
    v.status = green_status.p;
    launches += launch_green_solve(v, green_args(false), stream);
    MAG_CK(cudaGetLastError());
}

GreenArgs Sim::green_args(bool vacuum) const
{
    GreenArgs g{};
    g.G = green.p;
    g.u_vac = vacuum ? green_vac.p : nullptr;
    const long long nn = (long long)nx * nz;
    g.list_j = green_j.p;
    g.list_b = green_b.p;
    g.tile_count = green_j.p + nn;
    g.part = green_part.p;
    g.nchunks = green_chunks_n;
    if (vacuum && partial_rows && green_rows.p) {
        const long long ntiles = (nn + 1023) / 1024;
        g.rows = green_rows.p;
        g.row_count = green_rows.p + ntiles * 1024;
        g.charged = green_charged.p;
    }
    return g;
}

// the nodes a partial direct solve left out, from its right-hand side
void Sim::ensure_full_u()
{
    if (!u_partial) return;
    GreenArgs g = green_args(true);
    g.rows = nullptr;
    launches += launch_green_product(green_last, g, false, stream);
    if (green_last.Exf)
        launches += launch_faces(green_last.u, nx, nz, dx, dz, green_last.Exf, green_last.Ezf, stream);
    MAG_CK(cudaGetLastError());
    u_partial = false;
}

// Fields::u_smooth() where Pic::advance and Pic::advance_init call it
// (pic.cpp:336, 372): the whole potential, then the faces the push reads
void Sim::smooth_u()
{
    ensure_full_u();
    const size_t nn = (size_t)nx * nz;
    if (!u_tmp.p) u_tmp.alloc(nn);
    MAG_CK(cudaMemcpyAsync(u_tmp.p, u64.p, nn * sizeof(double), cudaMemcpyDeviceToDevice, stream));
    launches += launch_u_smooth(u_tmp.p, u64.p, nx, nz, stream);
    launches += launch_faces(u64.p, nx, nz, dx, dz, Exf.p, Ezf.p, stream);
    MAG_CK(cudaGetLastError());
}

void Sim::run_solve(SolveArgs a)
{
    u_partial = false;  // every path below writes u (a partial direct solve sets it again)
    if (mg_fp64) {
        MG64Args g{};
        for (int l = 0; l < lv.nlev; ++l) {
            g.lev[l].nx = lv.nx[l];
            g.lev[l].nz = lv.nz[l];
            g.lev[l].cmode = lv.cmode[l];
            g.lev[l].e = lv.e64[l].p;
            g.lev[l].r = lv.r64[l].p;
            g.lev[l].t = lv.t64[l].p;
            g.lev[l].coef = l > 0 ? lv.coef64[l].p : nullptr;
            g.lev[l].inv_diag = l > 0 ? lv.inv_diag64[l].p : nullptr;
        }
        g.coarse_inv = lv.coarse_inv64.p;
        launches += launch_solve64(a, g, stream);
        MAG_CK(cudaGetLastError());
        return;
    }
    if (a.rho_src != 3 && direct_mode >= 0 && p.selfconsistent && !a.rf_solve) {
        if (!green_tried) build_green();
        if (green_ready()) {
            // the stored electrode potential holds for this instance's own voltages
            const GreenArgs g = green_args(a.voltage == d_volt.p);
            launches += launch_green_solve(a, g, stream);
            MAG_CK(cudaGetLastError());
            u_partial = g.rows != nullptr;
            green_last = a;
            return;
        }
    }
    // grids above kSingleBlockNodes: one block of 1024 threads per SM under a
    // cooperative launch; their coarse levels below that size run on block 0
    int nblocks = 1;
    a.l_single = 0;
    a.tiled = 0;
    a.coarse_staged = 0;
    if ((long long)nx * nz > kSingleBlockNodes) {
        int ls = lv.nlev;
        for (int l = 0; l < lv.nlev; ++l)
            if ((long long)lv.nx[l] * lv.nz[l] <= kSingleBlockLevel) {
                ls = l;
                break;
            }
        if (solve_blocks == 0) {
            // tile phases on the levels above ls: one tile region per block in
            // shared memory (up to 200 KB), when the pre- and post-smoothing
            // passes fit the halo and the cooperative launch keeps one block per SM
            const long long smem_max = 200LL << 10;
            const int base_blocks = std::min(solve_max_blocks(sm_count), sm_count);
            const bool fits = ls > 0 && ls < lv.nlev && 2 * std::max(a.nu1, a.nu2) <= kTileHalo - 2;
            lv.ti.assign(lv.nlev, 0);
            lv.tj.assign(lv.nlev, 0);
            lv.staged.assign(lv.nlev, 0);
            lv.tile_smem = 0;
            if (fits && base_blocks > 1) {
                size_t smem = 0;
                for (int l = 0; l < ls; ++l) {
                    // a Galerkin level stages its operator with the tile when that
                    // still gives every block one tile; a larger level reads it from
                    // global memory and takes tiles of the fine level's size instead
                    // (fewer tile rounds, fewer halo nodes)
                    int bytes = kTileNodeBytes;
                    if (l > 0) {
                        int ti, tj;
                        choose_tile(lv.nx[l], lv.nz[l], base_blocks, kTileHalo, smem_max / kTileNodeBytesGalerkin, ti,
                                    tj);
                        const long long ntiles = (long long)((lv.nx[l] + ti - 1) / ti) * ((lv.nz[l] + tj - 1) / tj);
                        lv.staged[l] = ntiles <= base_blocks ? 1 : 0;
                        if (lv.staged[l]) bytes = kTileNodeBytesGalerkin;
                    }
                    choose_tile(lv.nx[l], lv.nz[l], base_blocks, kTileHalo, smem_max / bytes, lv.ti[l], lv.tj[l]);
                    smem = std::max(smem, (size_t)(lv.ti[l] + 2 * kTileHalo) * (lv.tj[l] + 2 * kTileHalo) * bytes);
                }
                // block 0's levels in shared memory: the arguments and 13 floats per node
                size_t stage = kStagedArgsBytes;
                for (int l = ls; l < lv.nlev; ++l) {
                    const size_t n = (size_t)lv.nx[l] * lv.nz[l];
                    stage += sizeof(float) * (4 * ((n + 3) & ~(size_t)3) + ((9 * n + 3) & ~(size_t)3));
                }
                const bool staged = stage <= (size_t)smem_max;
                if (staged) smem = std::max(smem, stage);
                if (std::min(solve_max_blocks(sm_count, smem), sm_count) >= base_blocks) {
                    lv.tile_smem = smem;
                    lv.coarse_staged = staged;
                }
            }
            solve_blocks = base_blocks;
        }
        nblocks = std::max(1, solve_blocks);
        if (nblocks > 1) {
            a.l_single = ls;
            a.coarse_grid = ls == lv.nlev - 1 && lv.coarse_inv_rows.p ? 1 : 0;
            if (lv.tile_smem) {
                a.tiled = 1;
                a.coarse_staged = lv.coarse_staged ? 1 : 0;
                for (int l = 0; l < ls; ++l) {
                    a.lev[l].ti = lv.ti[l];
                    a.lev[l].tj = lv.tj[l];
                    a.lev[l].staged = lv.staged[l];
                    const int tj = lv.tj[l], last = lv.nz[l] - (lv.nz[l] + tj - 1) / tj * tj + tj;
                    const int w[2] = {tj, last};
                    for (int c = 0; c < 2; ++c) {
                        a.lev[l].tw[c] = div_magic((unsigned)(w[c] + 2 * kTileHalo));
                        a.lev[l].th[c] = div_magic((unsigned)((w[c] + 2 * kTileHalo + 1) / 2));
                        a.lev[l].tn[c] = div_magic((unsigned)w[c]);
                    }
                }
            }
            MAG_CK(cudaMemsetAsync(d_bar.p, 0, sizeof(GridBarrier), stream));
            MAG_CK(cudaMemsetAsync(red.p, 0, 8 * sizeof(double), stream));
        }
    }
    if (a.prof) MAG_CK(cudaMemsetAsync(a.prof, 0, kSolvePhases * sizeof(double), stream));
    launches += launch_solve(a, nblocks, stream, a.tiled ? lv.tile_smem : 0);
    MAG_CK(cudaGetLastError());
}

// Arguments of one Poisson solve (Fields::boundary_solve / boundary_solve_rf)
SolveArgs Sim::solve_args(bool rf_solve, int rho_src, bool clear_rho)
{
    setup_solver();
    SolveArgs a{};
    a.coord = p.coord == CYLINDRICAL ? 1 : 0;
    a.nx = nx;
    a.nz = nz;
    a.dx = dx;
    a.dz = dz;
    a.mask = d_mask.p;
    a.voltage = d_volt.p;
    a.u = rf_solve ? urf64.p : u64.p;
    a.b = b64.p;
    a.rf_solve = rf_solve ? 1 : 0;
    a.rho_src = rho_src;
    a.nsp = (int)sp.size();
    for (size_t s = 0; s < sp.size(); ++s) {
        a.rho_fixed[s] = sp[s].rho.p;
        a.rho_weight[s] = sp[s].prm.charge * std::ldexp(1.0, -2 * kDepositShift);
    }
    a.rho64 = rho64.p;
    a.clear_rho = clear_rho ? 1 : 0;
    a.mpf = p.macroparticle_factor;
    a.dV = p.dV;
    a.st64 = lv.st64.p;
    a.rscale = lv.rscale.p;
    a.idx = 1.0 / dx;
    a.idz = 1.0 / dz;
    a.st32 = lv.st32.p;
    a.k2 = lv.k2;
    a.coarse_inv = lv.coarse_inv.p;
    a.coarse_inv_rows = lv.coarse_inv_rows.p;
    a.coarse_grid = 0;
    a.nlev = lv.nlev;
    for (int l = 0; l < lv.nlev; ++l) {
        a.lev[l].nx = lv.nx[l];
        a.lev[l].nz = lv.nz[l];
        a.lev[l].dz = div_magic((unsigned)lv.nz[l]);
        a.lev[l].dhz = div_magic((unsigned)((lv.nz[l] + 1) / 2));
        a.lev[l].e = lv.e[l].p;
        a.lev[l].r = lv.r[l].p;
        a.lev[l].t = lv.t[l].p;
        a.lev[l].coef = lv.coef[l].p;
        a.lev[l].inv_diag = lv.inv_diag[l].p;
        a.lev[l].cmode = lv.cmode[l];
    }
    a.nu1 = 2;
    a.nu2 = 2;
    a.ncoarse = lv.nlev == 1 ? 20 : 40;
    a.omega = lv.nlev == 1 ? (float)(2.0 / (1.0 + std::sin(kPi / std::max(nx, nz)))) : 1.f;
    a.tol = poisson_tol;
    a.max_outer = lv.nlev == 1 ? 20 * poisson_max_iter : poisson_max_iter;
    if (extrapolate_u && rho_src == 1 && clear_rho && !rf_solve) {
        // a step's solve starts from 2 u_n - u_(n-1)
        if (!u_prev.p) {
            u_prev.alloc((size_t)nx * nz);
            u_prev_valid.alloc(1);
            u_prev_valid.zero(stream);
        }
        a.u_prev = u_prev.p;
        a.u_prev_valid = u_prev_valid.p;
    }
    a.Exf = rf_solve ? Exf_rf.p : Exf.p;
    a.Ezf = rf_solve ? Ezf_rf.p : Ezf.p;
    a.red = red.p;
    a.bar = d_bar.p;
    a.status = d_status.p;
    a.err = d_err.p;
    a.prof = prof_on ? d_prof.p : nullptr;
    return a;
}

// Phase timing of the multigrid solve: on from the first call; the times of
// the most recent multigrid solve since then, in ms
int Sim::solve_phase_times(double* out, int cap)
{
    if (!prof_on) {
        d_prof.alloc(kSolvePhases);
        d_prof.zero(stream);
        prof_on = true;
    }
    std::vector<double> ns(kSolvePhases, 0.0);
    MAG_CK(cudaStreamSynchronize(stream));
    MAG_CK(cudaMemcpy(ns.data(), d_prof.p, kSolvePhases * sizeof(double), cudaMemcpyDeviceToHost));
    const int n = std::min(cap, kSolvePhases);
    for (int k = 0; k < n; ++k) out[k] = ns[k] * 1e-6;
    return n;
}

// Speclist (pic.cpp:27-80) and lifetime_init (particles.cpp:142-206)
void Sim::setup_species() { build_species(species_prm, inters, (size_t)nx * nz, stream, sp, d_inter, d_tables); }

// Species states, null-collision rates and the device interaction list of a
// species_conf (Speclist, src/pic.cpp:30-110): shared by the 2D and 3D runs.
void build_species(const std::vector<SpeciesParams>& species_prm, std::vector<InteractionParams>& inters,
                   size_t grid_nodes, cudaStream_t stream, std::vector<SpeciesState>& sp, DevArray<InterDev>& d_inter,
                   DevArray<double>& d_tables)
{
    const int ns = (int)species_prm.size();
    sp.resize(ns);
    std::map<std::string, int> idx;
    for (int s = 0; s < ns; ++s) idx[species_prm[s].name] = s;
    for (int s = 0; s < ns; ++s) {
        SpeciesState& S = sp[s];
        S.prm = species_prm[s];
        S.E_max = S.prm.E_max > 0. ? S.prm.E_max : S.prm.temperature * kKB / kQe * 10.0;
        S.v_max = std::sqrt(2.0 * kKB * S.prm.temperature / S.prm.mass);
        S.by_target.assign(ns, {});
        S.rates.assign(ns, 0.0);
        S.cnt.alloc(1);
        S.cnt.zero(stream);
        S.rho.alloc(grid_nodes);
        S.rho.zero(stream);
    }
    std::vector<InterDev> idev;
    std::vector<double> tab;
    const std::vector<InteractionParams> raw_inters = inters;
    for (size_t q = 0; q < inters.size(); ++q) {
        const InteractionParams& in = inters[q];
        auto pi = idx.find(in.primary), si = idx.find(in.secondary);
        if (pi == idx.end())
            throw Error(-1, "Speclist::Speclist: unrecognized primary species \"" + in.primary + "\" of interaction \"" +
                                in.name + "\"");
        if (si == idx.end())
            throw Error(-1, "Speclist::Speclist: unrecognized primary species \"" + in.secondary +
                                "\" of interaction \"" + in.name + "\"");
        sp[pi->second].by_target[si->second].push_back((int)q);
        if (in.type == LANGEVIN) inters[q].rate *= in.cutoff * in.cutoff;  // particles.hpp:81-82
    }
    for (int s = 0; s < ns; ++s) {
        SpeciesState& S = sp[s];
        species_rates(species_prm, raw_inters, s, S.rates, S.lifetime);
        S.prob = 1.0 - std::exp(-S.prm.dt / S.lifetime);
        const double th = S.prob * 4294967296.0;
        S.threshold = S.prob <= 0.0 ? 0u : (th >= 4294967295.0 ? 0xffffffffu : (uint32_t)std::max(1.0, th));
    }
    // device interaction list grouped per primary species, then per target,
    // in the order of the species_conf file (interactions_by_species)
    auto make_dev = [&](int q) {
        const InteractionParams& in = inters[q];
        const int pr = idx[in.primary], se = idx[in.secondary];
        InterDev d{};
        d.type = in.type;
        d.target = se;
        d.DE = in.DE * kQe;
        d.rate = in.rate;
        d.cutoff = in.cutoff;
        const double m1 = species_prm[pr].mass, m2 = species_prm[se].mass;
        d.mu = m1 * m2 / (m1 + m2);
        d.tab_off = (int)tab.size();
        d.tab_n = (int)in.CS_energy.size();
        tab.insert(tab.end(), in.CS_energy.begin(), in.CS_energy.end());
        tab.insert(tab.end(), in.CS_value.begin(), in.CS_value.end());
        const SpeciesParams& P = species_prm[pr];
        d.coul_lambda_D = std::sqrt(kEps0 * kKB * P.temperature / (P.density * P.charge * P.charge));
        d.coul_q1q2 = P.charge * species_prm[se].charge;
        return d;
    };
    for (int s = 0; s < ns; ++s) {
        sp[s].inter_off = (int)idev.size();
        for (int t = 0; t < ns; ++t)
            for (int q : sp[s].by_target[t]) idev.push_back(make_dev(q));
    }
    if (idev.empty()) idev.push_back(InterDev{});
    if (tab.empty()) tab.push_back(0.0);
    d_inter.upload(idev.data(), idev.size(), stream);
    d_tables.upload(tab.data(), tab.size(), stream);
    for (int s = 0; s < ns; ++s) {
        SpeciesState& S = sp[s];
        MccSpecies m{};
        m.mass = S.prm.mass;
        m.inv_lifetime = std::isinf(S.lifetime) ? 0.0 : 1.0 / S.lifetime;
        m.nsp = ns;
        int pos = S.inter_off;
        for (int t = 0; t < ns; ++t) {
            m.rates[t] = S.rates[t];
            m.t_mass[t] = species_prm[t].mass;
            m.t_density[t] = species_prm[t].density;
            m.t_sigma_v[t] = std::sqrt(2.0 * kKB * species_prm[t].temperature / species_prm[t].mass) * std::sqrt(0.5);
            m.inter_begin[t] = pos;
            pos += (int)S.by_target[t].size();
            m.inter_end[t] = pos;
        }
        m.inter = d_inter.p;
        m.tables = d_tables.p;
        S.mcc.upload(&m, 1, stream);
    }
    MAG_CK(cudaStreamSynchronize(stream));
}

void Sim::ensure_capacity(int s, int64_t need)
{
    SpeciesState& S = sp[s];
    if (need <= S.cap) return;
    int64_t cap = std::max<int64_t>(need, (int64_t)(S.cap * 1.5) + 1024);
    cap = (cap + kSlotAlign - 1) / kSlotAlign * kSlotAlign;  // whole vector groups
    MAG_CK(cudaStreamSynchronize(stream));
    auto grow = [&](auto& a) {
        typename std::remove_reference<decltype(a)>::type b;
        b.alloc(cap);
        if (S.n_slots)
            MAG_CK(cudaMemcpyAsync(b.p, a.p, S.n_slots * sizeof(*a.p), cudaMemcpyDeviceToDevice, stream));
        MAG_CK(cudaStreamSynchronize(stream));
        a = std::move(b);
    };
    grow(S.x);
    grow(S.z);
    grow(S.vx);
    grow(S.vy);
    grow(S.vz);
    grow(S.id);
    S.cand.alloc(cap);
    S.cand_rec.alloc(cap);
    if (multicoll) grow(S.ttd);
    S.bx.release();  // sort buffers are re-made at the next sort
    S.bz.release();
    S.bvx.release();
    S.bvy.release();
    S.bvz.release();
    S.bid.release();
    S.cap = cap;
}

void Sim::add_loaded(int s, int64_t n, int kind, double cx, double cz, double radius, double zlo, double zhi)
{
    if (n <= 0) return;
    SpeciesState& S = sp[s];
    ensure_capacity(s, S.n_slots + n);
    const double vsig = S.v_max * std::sqrt(0.5);
    const int64_t o = S.n_slots;
    launches += launch_load_disk(S.x.p + o, S.z.p + o, S.vx.p + o, S.vy.p + o, S.vz.p + o, S.id.p + o, n, S.next_id,
                                 kind, cx, cz, radius, zlo, zhi, x0, z0, dx, dz, xmax, zmax, vsig, seed,
                                 (uint32_t)s, p.coord, stream);
    MAG_CK(cudaGetLastError());
    S.n_slots += n;
    S.next_id += (uint32_t)n;
    S.scrambled = true;
    upload_slots(s);
    init_ttd(s, o, n);
    sort_due = true;
}

// time_to_death = lifetime * rexp of new particles (add_particles_*, src/particles.cpp:697)
void Sim::init_ttd(int s, int64_t first, int64_t n)
{
    if (!multicoll || n <= 0) return;
    SpeciesState& S = sp[s];
    launches += launch_init_ttd(S.ttd.p, S.id.p, first, n, S.lifetime, seed, (uint32_t)s, S.niter, stream);
    MAG_CK(cudaGetLastError());
}

void Sim::add_single(int s, double x, double z, double vx, double vy, double vz)
{
    SpeciesState& S = sp[s];
    ensure_capacity(s, S.n_slots + 1);
    const int64_t o = S.n_slots;
    const bool inside = x >= x0 && x <= xmax && z >= z0 && z <= zmax;
    uint32_t fx = inside ? (uint32_t)std::llrint((x - x0) / dx * (double)(1u << kFracBits)) : kDead;
    uint32_t fz = inside ? (uint32_t)std::llrint((z - z0) / dz * (double)(1u << kFracBits)) : 0u;
    float fvx = (float)vx, fvy = (float)vy, fvz = (float)vz;
    uint32_t pid = S.next_id;
    MAG_CK(cudaMemcpy(S.x.p + o, &fx, 4, cudaMemcpyHostToDevice));
    MAG_CK(cudaMemcpy(S.z.p + o, &fz, 4, cudaMemcpyHostToDevice));
    MAG_CK(cudaMemcpy(S.vx.p + o, &fvx, 4, cudaMemcpyHostToDevice));
    MAG_CK(cudaMemcpy(S.vy.p + o, &fvy, 4, cudaMemcpyHostToDevice));
    MAG_CK(cudaMemcpy(S.vz.p + o, &fvz, 4, cudaMemcpyHostToDevice));
    MAG_CK(cudaMemcpy(S.id.p + o, &pid, 4, cudaMemcpyHostToDevice));
    S.n_slots += 1;
    S.next_id += 1;
    upload_slots(s);
    init_ttd(s, o, 1);
    sort_due = true;
}

// Pic::run_initscript (src/pic.cpp:241-328) plus one r-z loader
void Sim::run_initscript(const std::string& path)
{
    std::ifstream fr(path);
    if (!fr) throw Error(-6, "cannot open initscript " + path);
    std::map<std::string, int> idx;
    for (size_t s = 0; s < species_prm.size(); ++s) idx[species_prm[s].name] = (int)s;
    auto species = [&](const std::string& name) {
        auto it = idx.find(name);
        if (it == idx.end()) throw Error(-1, "Pic::run_initscript: unrecognized species type \"" + name + "\"");
        return it->second;
    };
    std::string line;
    while (std::getline(fr, line)) {
        if (!line.empty() && line[0] == '#') continue;
        std::vector<std::string> t = tokens(line);
        if (t.empty()) continue;
        auto need = [&](size_t k) {
            if (t.size() != k)
                throw Error(-1, "Pic::run_initscript: wrong number of parameters (" + std::to_string(t.size()) +
                                    ") to " + t[0]);
        };
        const bool cyl = p.coord == CYLINDRICAL;
        if (t[0] == "add_particles_bessel" || t[0] == "add_particles_everywhere" || t[0] == "add_particles_on_disk") {
            if (cyl) throw Error(-1, t[0] + " is not defined for CYLINDRICAL in the reference");
        }
        if (t[0] == "add_particles_bessel") {
            need(6);
            add_loaded(species(t[1]), to_int(t[2]), 2, to_num(t[3]), to_num(t[4]), to_num(t[5]), 0, 0);
        } else if (t[0] == "add_particles_everywhere") {
            need(3);
            add_loaded(species(t[1]), to_int(t[2]), 1, 0, 0, 0, 0, 0);
        } else if (t[0] == "add_particles_on_disk") {
            need(6);
            add_loaded(species(t[1]), to_int(t[2]), 0, to_num(t[3]), to_num(t[4]), to_num(t[5]), 0, 0);
        } else if (t[0] == "add_tracked_particle") {
            need(7);  // particles.hpp:297-309: y and z components are swapped on input
            const int s = species(t[1]);
            tracked.push_back({s, sp[s].next_id, sp[s].n_slots, nullptr});
            add_single(s, to_num(t[2]), to_num(t[3]), to_num(t[4]), to_num(t[6]), to_num(t[5]));
        } else if (t[0] == "add_particles_in_cylinder") {
            // r-z loader: species n r_max z_min z_max, uniform in volume (r = r_max sqrt(u))
            need(6);
            if (!cyl) throw Error(-1, "add_particles_in_cylinder needs coord = CYLINDRICAL");
            add_loaded(species(t[1]), to_int(t[2]), 3, 0, 0, to_num(t[3]), to_num(t[4]), to_num(t[5]));
        }
    }
    MAG_CK(cudaStreamSynchronize(stream));
}

PushArgs Sim::push_args(int s, bool init)
{
    SpeciesState& S = sp[s];
    PushArgs a{};
    a.x = S.x.p;
    a.z = S.z.p;
    a.vx = S.vx.p;
    a.vy = S.vy.p;
    a.vz = S.vz.p;
    a.id = S.id.p;
    a.n = S.n_slots;
    a.n_dev = &S.cnt.p->slots;
    a.nx = nx;
    a.nz = nz;
    a.xmaxf = (uint32_t)std::llrint((xmax - x0) / dx * (double)(1u << kFracBits));
    a.zmaxf = (uint32_t)std::llrint((zmax - z0) / dz * (double)(1u << kFracBits));
    a.periodic = p.boundary == BND_PERIODIC ? 1 : 0;
    a.check_mask = check_mask ? 1 : 0;
    a.mask = d_mask.p;
    a.cellfree = d_cellfree.p;
    a.emode = emode;
    a.Exf = Exf.p;
    a.Ezf = Ezf.p;
    a.Exf2 = Exf2.p;
    a.Ezf2 = Ezf2.p;
    a.extern_ez = (float)p.extern_field;
    a.step = S.niter;
    a.phase = rf_factor(S.niter, S.prm.dt);
    const double q = S.prm.charge, m = S.prm.mass, dt = S.prm.dt;
    const double rot = init ? -0.5 * q * dt / (2.0 * m) : q * dt / (2.0 * m);
    a.q_dt_2m = (float)rot;
    a.hq = (float)(init ? -q / m * dt / 2.0 : q / m * dt / 2.0);
    const double tx = p.Br * rot, ty = p.Bt * rot, tz = p.Bz * rot;
    const double f = 2.0 / (1 + tx * tx + ty * ty + tz * tz);
    auto split = [](double v, float& hi, float& lo) {
        hi = (float)v;
        lo = (float)(v - (double)hi);
    };
    split(tx, a.tx, a.tlx);
    split(ty, a.ty, a.tly);
    split(tz, a.tz, a.tlz);
    split(tx * f, a.sx, a.slx);
    split(ty * f, a.sy, a.sly);
    split(tz * f, a.sz, a.slz);
    a.btab = p.magnetic_field_const ? 0 : 1;
    a.has_b = (a.btab || p.Br != 0.0 || p.Bt != 0.0 || p.Bz != 0.0) ? 1 : 0;
    a.Br = d_Br.p;
    a.Bz = d_Bz.p;
    a.bnx = bnx;
    a.bnz = bnz;
    a.b_x0 = (float)b_x0;
    a.b_z0 = (float)b_z0;
    a.b_ix = (float)(1.0 / b_dx);
    a.b_iz = (float)(1.0 / b_dz);
    a.gdx = (float)dx;
    a.gdz = (float)dz;
    a.gx0 = (float)x0;
    a.gz0 = (float)z0;
    a.cx = (float)(dt / dx);
    a.cz = (float)(dt / dz);
    a.rho = p.selfconsistent ? S.rho.p : nullptr;
    a.coll_threshold = init ? 0u : S.threshold;
    a.cand = S.cand.p;
    a.cand_rec = S.cand_rec.p;
    a.mcc = S.mcc.p;
    a.seed = seed;
    a.species = (uint32_t)s;
    a.cnt = S.cnt.p;
    a.slot = 0;
    a.fold_slot = -1;
    return a;
}

// Fields::E phase at t = niter * dt, in FP64 as the reference (fields.hpp:135-145)
float Sim::rf_factor(uint64_t niter, double dt) const
{
    const double t = (double)niter * dt;
    double ph = p.rf_omega * t;
    const double y = 10000000 * kPi;
    if (!(ph >= 0.0 && ph <= y)) ph = ph - y * (double)(int)(ph / y) + (ph < 0 ? y : 0);
    return (float)(p.rf_amplitude * std::cos(ph) + p.rf_U0);
}

// 0: no collisions; 2: the particle kernel lists candidates, k_collide runs them
int Sim::coll_mode(int s) const { return sp[s].threshold == 0 ? 0 : 2; }

bool Sim::any_target_slots(int s) const
{
    const SpeciesState& S = sp[s];
    for (size_t t = 0; t < sp.size() && t < S.rates.size(); ++t)
        if (S.rates[t] > 0.0 && sp[t].n_slots > 0) return true;
    return false;
}

CollideArgs Sim::collide_args(int s)
{
    SpeciesState& S = sp[s];
    CollideArgs a{};
    a.vx = S.vx.p;
    a.vy = S.vy.p;
    a.vz = S.vz.p;
    a.cand = S.cand.p;
    a.cand_rec = S.cand_rec.p;
    a.cnt = S.cnt.p;
    a.mcc = S.mcc.p;
    a.inter = d_inter.p;
    a.n_inter = (int)d_inter.n;
    a.tables = d_tables.p;
    a.n_tables = (int)d_tables.n;
    for (size_t t = 0; t < sp.size(); ++t) {
        a.t_has_slots[t] = sp[t].n_slots > 0 ? 1 : 0;
        a.t_x[t] = sp[t].x.p;
        a.t_vx[t] = sp[t].vx.p;
        a.t_vy[t] = sp[t].vy.p;
        a.t_vz[t] = sp[t].vz.p;
        a.t_n[t] = sp[t].n_slots;
    }
    a.any_target_slots = any_target_slots(s) ? 1 : 0;
    a.seed = seed;
    a.species = (uint32_t)s;
    a.step = S.niter;
    return a;
}

// Counting sort by cell into the double buffers, then swap (compacts removed particles).
// Counting sort of one species by cell.  Slots that a loader or
// set_particles filled in no cell order are sorted in three passes of
// decreasing key size (blocks of 64 x 128 cells, blocks of 4 x 8 cells, cells),
// so that each pass meets only a few hundred keys per chunk of slots and its
// stores leave in runs; slots sorted a few steps ago take the single pass by cell.
void Sim::sort_species(int s)
{
    SpeciesState& S = sp[s];
    if (S.n_slots == 0 || multicoll) return;  // the uniform field has no gather to keep local
    if (!S.bx.p) {
        S.bx.alloc(S.cap);
        S.bz.alloc(S.cap);
        S.bvx.alloc(S.cap);
        S.bvy.alloc(S.cap);
        S.bvz.alloc(S.cap);
        S.bid.alloc(S.cap);
    }
    struct KeyLevel {
        int si, sj;
    };
    static const KeyLevel kScrambled[3] = {{6, 7}, {2, 3}, {0, 0}};
    static const KeyLevel kCells[1] = {{0, 0}};
    const bool three = S.scrambled && S.n_slots >= kScrambledSortMin;
    const KeyLevel* lv = three ? kScrambled : kCells;
    for (int pass = 0; pass < (three ? 3 : 1); ++pass) {
        SortArgs a{};
        a.x = S.x.p;
        a.z = S.z.p;
        a.vx = S.vx.p;
        a.vy = S.vy.p;
        a.vz = S.vz.p;
        a.id = S.id.p;
        a.ox = S.bx.p;
        a.oz = S.bz.p;
        a.ovx = S.bvx.p;
        a.ovy = S.bvy.p;
        a.ovz = S.bvz.p;
        a.oid = S.bid.p;
        a.n = S.n_slots;
        a.nx = nx;
        a.nz = nz;
        a.si = lv[pass].si;
        a.sj = lv[pass].sj;
        a.nzk = ((nz - 2) >> a.sj) + 1;
        a.ncells = (long long)(((nx - 2) >> a.si) + 1) * a.nzk;
        a.count = sort_count.p;
        a.offset = sort_offset.p;
        a.blocksum = sort_blocksum.p;
        a.cnt = S.cnt.p;
        launches += launch_sort(a, S.n_slots, stream);
        std::swap(S.x, S.bx);
        std::swap(S.z, S.bz);
        std::swap(S.vx, S.bvx);
        std::swap(S.vy, S.bvy);
        std::swap(S.vz, S.bvz);
        std::swap(S.id, S.bid);
    }
    S.scrambled = false;
}

// One Pic::advance (src/pic.cpp:330-358).  Species advance in order, each
// with its collisions (as Species::advance runs scatter inside the push loop).
// With ms != nullptr, events split the step into sort, solve, particle
// kernels and collision kernels and the four device times are added to ms
// (an event between a particle kernel and its collision kernel removes their
// overlap, so the split costs a little time).
void Sim::step(double* ms)
{
    std::vector<cudaEvent_t> ev;
    std::vector<int> kind;  // window of the interval that ends at each event
    auto mark = [&](int k) {
        if (!ms) return;
        cudaEvent_t e;
        MAG_CK(cudaEventCreate(&e));
        MAG_CK(cudaEventRecord(e, stream));
        ev.push_back(e);
        kind.push_back(k);
    };
    mark(-1);
    if (sort_interval > 0 && (sort_due || steps_done % (uint64_t)sort_interval == 0)) {
        for (size_t s = 0; s < sp.size(); ++s) sort_species((int)s);
        sort_due = false;
    }
    ++steps_done;
    mark(0);
    if (p.selfconsistent) {
        solve(false, rho_override ? 2 : 1, true, false);
        if (p.u_smooth) smooth_u();
    }
    rho_override = false;
    mark(1);
    for (size_t s = 0; s < sp.size(); ++s) {
        SpeciesState& S = sp[s];
        if (S.n_slots == 0) {
            S.niter++;
            continue;
        }
        PushArgs pa = push_args((int)s, false);
        pa.slot = (int)(S.launches & 1);
        pa.fold_slot = S.launches > 0 ? (int)((S.launches - 1) & 1) : -1;
        if (multicoll) {  // event-driven mover, collisions inside the kernel
            const CollideArgs ca = collide_args((int)s);
            if (ca.any_target_slots)
                throw Error(-1, "ADVANCE_MULTICOLL: collision partners must be background species (no particles)");
            launches += launch_multicoll(pa, ca, S.ttd.p, S.prm.dt, S.lifetime, S.prm.charge / S.prm.mass, stream);
            mark(2);
            S.launches++;
            S.niter++;
            continue;
        }
        launches += launch_push(pa, p.coord == CYLINDRICAL ? 1 : 0, false, push_vec_for(S.n_slots), sm_count, stream);
        mark(2);
        if (coll_mode((int)s) == 2) {
            CollideArgs ca = collide_args((int)s);
            ca.slot = pa.slot;
            const double expect = (double)S.n_slots * S.prob;
            const int grid = (int)std::min<double>(4.0 * sm_count, std::ceil(4.0 * expect / 128.0) + 1.0);
            launches += launch_collide(ca, grid, stream);
            mark(3);
        }
        S.launches++;
        S.niter++;
        if (p.use_source) source_step((int)s);  // Pic::advance (src/pic.cpp:344-348)
    }
    if (ms) {
        MAG_CK(cudaEventSynchronize(ev.back()));
        for (size_t k = 1; k < ev.size(); ++k) {
            float t = 0.f;
            MAG_CK(cudaEventElapsedTime(&t, ev[k - 1], ev[k]));
            ms[kind[k]] += t;
        }
        for (auto e : ev) cudaEventDestroy(e);
    }
}

// Particles are independent over the next steps when nothing couples them:
// no self-consistent field, the per-step mover (not ADVANCE_MULTICOLL) and
// collision targets without particles.  The block ends before the next sort.
int Sim::fused_steps(uint64_t left) const
{
    if (max_fused <= 1 || left <= 1 || p.selfconsistent || multicoll || p.use_source) return 1;
    for (size_t s = 0; s < sp.size(); ++s)
        if (sp[s].n_slots > 0 && coll_mode((int)s) != 0 && any_target_slots((int)s)) return 1;
    uint64_t k = std::min<uint64_t>(left, (uint64_t)max_fused);
    if (sort_interval > 0) k = std::min<uint64_t>(k, (uint64_t)sort_interval - steps_done % (uint64_t)sort_interval);
    return (int)std::max<uint64_t>(k, 1);
}

// nsteps steps of every species as one launch per species (k_push_fused);
// the same sort, counters and step counters as nsteps calls of step()
void Sim::fused_block(int nsteps, double* ms)
{
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    if (ms)
        for (auto& e : ev) {
            MAG_CK(cudaEventCreate(&e));
        }
    if (ms) MAG_CK(cudaEventRecord(ev[0], stream));
    if (sort_interval > 0 && (sort_due || steps_done % (uint64_t)sort_interval == 0)) {
        for (size_t s = 0; s < sp.size(); ++s) sort_species((int)s);
        sort_due = false;
    }
    if (ms) MAG_CK(cudaEventRecord(ev[1], stream));
    steps_done += (uint64_t)nsteps;
    rho_override = false;
    for (size_t s = 0; s < sp.size(); ++s) {
        SpeciesState& S = sp[s];
        if (S.n_slots == 0) {
            S.niter += (uint64_t)nsteps;
            continue;
        }
        PushArgs pa = push_args((int)s, false);
        pa.slot = (int)(S.launches & 1);
        pa.fold_slot = S.launches > 0 ? (int)((S.launches - 1) & 1) : -1;
        const CollideArgs ca = coll_mode((int)s) == 2 ? collide_args((int)s) : CollideArgs{};
        FusedSteps fs{};
        fs.nsteps = nsteps;
        for (int q = 0; q < nsteps; ++q) fs.phase[q] = rf_factor(S.niter + (uint64_t)q, S.prm.dt);
        launches += launch_push_fused(pa, ca, fs, p.coord == CYLINDRICAL ? 1 : 0, sm_count, stream);
        S.launches++;
        S.niter += (uint64_t)nsteps;
    }
    if (ms) {
        MAG_CK(cudaEventRecord(ev[2], stream));
        MAG_CK(cudaEventSynchronize(ev[2]));
        float t0 = 0.f, t1 = 0.f;
        MAG_CK(cudaEventElapsedTime(&t0, ev[0], ev[1]));
        MAG_CK(cudaEventElapsedTime(&t1, ev[1], ev[2]));
        ms[0] += t0;
        ms[2] += t1;
        for (auto e : ev) cudaEventDestroy(e);
    }
}

void Sim::advance_timed(uint64_t nsteps, double* ms4)
{
    MAG_CK(cudaSetDevice(device));
    for (int k = 0; k < 4; ++k) ms4[k] = 0.0;
    for (uint64_t left = nsteps; left > 0;) {
        const int k = fused_steps(left);
        if (k > 1) fused_block(k, ms4);
        else step(ms4);
        left -= (uint64_t)k;
    }
}

void Sim::advance(uint64_t nsteps)
{
    MAG_CK(cudaSetDevice(device));
    for (uint64_t left = nsteps; left > 0;) {
        const int k = fused_steps(left);
        if (k > 1) fused_block(k);
        else step();
        left -= (uint64_t)k;
    }
    MAG_CK(cudaGetLastError());
}

// Pic::advance_init (src/pic.cpp:359-384)
void Sim::advance_init(bool deposit)
{
    MAG_CK(cudaSetDevice(device));
    if (p.selfconsistent) {
        if (deposit) deposit_all();
        solve(false, 1, false, false);
        if (p.u_smooth) smooth_u();
    }
    for (size_t s = 0; s < sp.size(); ++s) {
        if (sp[s].n_slots == 0 || multicoll) continue;  // ADVANCE_MULTICOLL has no leapfrog start
        PushArgs pa = push_args((int)s, true);
        launches += launch_push(pa, p.coord == CYLINDRICAL ? 1 : 0, true, push_vec_for(sp[s].n_slots), sm_count, stream);
    }
    if (p.use_source) source_refresh(p.src_fact);  // the driver's refresh after advance_init (src/test.cpp:56-59)
    MAG_CK(cudaGetLastError());
}

void Sim::deposit_all()
{
    for (size_t s = 0; s < sp.size(); ++s) {
        sp[s].rho.zero(stream);
        if (sp[s].n_slots == 0) continue;
        PushArgs pa = push_args((int)s, false);
        pa.rho = sp[s].rho.p;
        launches += launch_deposit(pa, stream);
    }
    rho_override = false;
}

SolveStatus Sim::field_solve()
{
    if (p.electric_field_from_file)
        throw Error(-1, "no Poisson solve with electric_field_from_file (the reference forbids it, param.cpp:62-64)");
    return solve(false, rho_override ? 2 : 1, false, true);
}

void Sim::get_faces(int component, float* out)
{
    ensure_full_u();
    const size_t n = component == 0 ? (size_t)(nx + 1) * nz : (size_t)nx * (nz + 1);
    MAG_CK(cudaStreamSynchronize(stream));
    MAG_CK(cudaMemcpy(out, component == 0 ? Exf.p : Ezf.p, n * sizeof(float), cudaMemcpyDeviceToHost));
}

void Sim::get_field(int which, double* out)
{
    const size_t nn = (size_t)nx * nz;
    if (which == 0) ensure_full_u();
    MAG_CK(cudaStreamSynchronize(stream));
    if (which == 0) u64.download(out, nn, stream);
    else if (which == 1) urf64.download(out, nn, stream);
    else if (which == 3) {
        for (size_t k = 0; k < mask.size(); ++k) out[k] = mask[k];
        return;
    } else if (which == 4) {
        std::copy(voltage.begin(), voltage.end(), out);
        return;
    } else if (which == 2 && rho_override) {
        rho64.download(out, nn, stream);
    } else if (which == 2 || which >= 5) {
        std::fill(out, out + nn, 0.0);
        std::vector<int64_t> acc(nn);
        const size_t s0 = which == 2 ? 0 : (size_t)(which - 5), s1 = which == 2 ? sp.size() : s0 + 1;
        if (s0 >= sp.size()) throw Error(-1, "species index out of range");
        for (size_t s = s0; s < s1; ++s) {
            MAG_CK(cudaMemcpyAsync(acc.data(), sp[s].rho.p, nn * 8, cudaMemcpyDeviceToHost, stream));
            MAG_CK(cudaStreamSynchronize(stream));
            const double w = sp[s].prm.charge * std::ldexp(1.0, -2 * kDepositShift);
            for (size_t k = 0; k < nn; ++k) out[k] += w * (double)acc[k];
        }
        return;
    } else
        throw Error(-1, "unknown field selector");
    MAG_CK(cudaStreamSynchronize(stream));
}

void Sim::set_field(int which, const double* in)
{
    const size_t nn = (size_t)nx * nz;
    if (which == 0) u_partial = false;
    if (which == 0 && u_prev_valid.p) u_prev_valid.zero(stream);  // no history for the next extrapolation
    if (which == 0) u64.upload(in, nn, stream);
    else if (which == 1) urf64.upload(in, nn, stream);
    else if (which == 2) {
        rho64.upload(in, nn, stream);
        rho_override = true;
    } else
        throw Error(-1, "only u, uRF and rho can be set");
    if (which == 0) launches += launch_faces(u64.p, nx, nz, dx, dz, Exf.p, Ezf.p, stream);
    if (which == 1) launches += launch_faces(urf64.p, nx, nz, dx, dz, Exf_rf.p, Ezf_rf.p, stream);
    if (which <= 1) refresh_rf_pairs();
    MAG_CK(cudaStreamSynchronize(stream));
}

void Sim::get_particles(int s, int64_t cap, double* x, double* z, double* vx, double* vy, double* vz, uint32_t* id,
                        int64_t* n_out)
{
    SpeciesState& S = sp[s];
    const int64_t n = S.n_slots;
    std::vector<uint32_t> hx(n), hz(n), hid(n);
    std::vector<float> hvx(n), hvy(n), hvz(n);
    S.x.download(hx.data(), n, stream);
    S.z.download(hz.data(), n, stream);
    S.vx.download(hvx.data(), n, stream);
    S.vy.download(hvy.data(), n, stream);
    S.vz.download(hvz.data(), n, stream);
    S.id.download(hid.data(), n, stream);
    MAG_CK(cudaStreamSynchronize(stream));
    int64_t m = 0;
    const double inv = 1.0 / (double)(1u << kFracBits);
    for (int64_t k = 0; k < n && m < cap; ++k) {
        if (hx[k] == kDead) continue;
        if (x) x[m] = x0 + (double)hx[k] * inv * dx;
        if (z) z[m] = z0 + (double)hz[k] * inv * dz;
        if (vx) vx[m] = hvx[k];
        if (vy) vy[m] = hvy[k];
        if (vz) vz[m] = hvz[k];
        if (id) id[m] = hid[k];
        ++m;
    }
    *n_out = m;
}

// The device address of a page-locked (cudaHostAlloc / cudaHostRegister) host
// array registered with this device, which kernels can read in place; false
// for any other memory
static bool host_mapped(const void* ptr, int device, const double** dev)
{
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess) {
        (void)cudaGetLastError();  // clear the error of an unknown pointer
        return false;
    }
    if (a.type != cudaMemoryTypeHost || a.devicePointer == nullptr || a.device != device) return false;
    *dev = static_cast<const double*>(a.devicePointer);
    return true;
}

void Sim::set_particles(int s, int64_t n, const double* x, const double* z, const double* vx, const double* vy,
                        const double* vz)
{
    SpeciesState& S = sp[s];
    S.n_slots = 0;
    ensure_capacity(s, std::max<int64_t>(n, 1));
    // the conversion to the fixed-point SoA runs on the device: it reads
    // page-locked host arrays in place, other arrays from a device staging
    // copy (the stream is synchronised below, so the caller's arrays are no
    // longer read when this returns)
    const double* src[5] = {x, z, vx, vy, vz};
    ParticleColumns cols{};
    bool mapped = n > 0;
    for (int c = 0; c < 5 && mapped; ++c) mapped = host_mapped(src[c], device, &cols.v[c]);
    if (!mapped) {
        if (stage64.n < (size_t)(5 * n)) stage64.alloc((size_t)(5 * n));
        for (int c = 0; c < 5; ++c) {
            cols.v[c] = stage64.p + (size_t)c * n;
            if (n) MAG_CK(cudaMemcpyAsync(stage64.p + (size_t)c * n, src[c], (size_t)n * sizeof(double),
                                          cudaMemcpyHostToDevice, stream));
        }
    }
    const SetParticlesGeom g{x0, xmax, z0, zmax, dx, dz};
    launches += launch_set_particles(cols, n, g, S.x.p, S.z.p, S.vx.p, S.vy.p, S.vz.p, S.id.p, stream);
    S.n_slots = n;
    S.next_id = (uint32_t)n;
    S.scrambled = cell_order_broken(x, z, n);
    upload_slots(s);
    init_ttd(s, 0, n);
    // particles read back from a sorted run keep the order the particle
    // kernel's deposit tiles rely on: only scrambled ones are sorted at once
    if (S.scrambled) sort_due = true;
}

// Whether host particles come in no cell order: eight windows of 512
// consecutive particles spread over the arrays, scrambled when more than a
// quarter of the neighbour pairs lie more than four grid rows apart.
// (Particles read back from a sorted run have moved a cell or two since:
// their neighbours stay within a few cells, while random order puts them a
// third of the grid apart.)
bool Sim::cell_order_broken(const double* x, const double* z, int64_t n) const
{
    if (n < 2) return false;
    auto index = [](double f, int last) {  // floor(f) clamped to [0, last]; non-finite -> 0
        return f >= 0.0 ? (int64_t)std::min(std::floor(f), (double)last) : (int64_t)0;
    };
    auto cell = [&](int64_t k) { return index((x[k] - x0) / dx, nx - 2) * (nz - 1) + index((z[k] - z0) / dz, nz - 2); };
    const int64_t w = std::min<int64_t>(512, n);
    const int64_t far = 4 * (int64_t)(nz - 1);
    int64_t pairs = 0, apart = 0;
    for (int k = 0; k < 8; ++k) {
        const int64_t first = (n - w) * k / 8;
        int64_t prev = cell(first);
        for (int64_t q = first + 1; q < first + w; ++q) {
            const int64_t c = cell(q);
            apart += std::llabs(c - prev) > far;
            ++pairs;
            prev = c;
        }
    }
    return 4 * apart > pairs;
}

// Pic::print_trace (src/pic.cpp:446-451): TrackedParticle::print of every
// tracked particle (particles.cpp:12-17), found by its id
void Sim::print_trace(const std::string& dir)
{
    if (tracked.empty()) return;
    const double inv = 1.0 / (double)(1u << kFracBits);
    for (size_t s = 0; s < sp.size(); ++s) {
        std::vector<uint32_t> want;
        std::vector<size_t> which;
        for (size_t k = 0; k < tracked.size(); ++k)
            if (tracked[k].s == (int)s) {
                want.push_back(tracked[k].id);
                which.push_back(k);
            }
        if (want.empty()) continue;
        SpeciesState& S = sp[s];
        const int nw = (int)want.size();
        DevArray<uint32_t> d_want, d_rec;
        d_want.upload(want.data(), want.size(), stream);
        d_rec.alloc((size_t)nw * 6);
        MAG_CK(cudaMemsetAsync(d_rec.p, 0, (size_t)nw * 6 * sizeof(uint32_t), stream));
        launches += launch_find_ids(S.id.p, S.x.p, S.z.p, S.vx.p, S.vy.p, S.vz.p, S.n_slots, d_want.p, nw, d_rec.p,
                                    stream);
        std::vector<uint32_t> rec((size_t)nw * 6);
        d_rec.download(rec.data(), rec.size(), stream);
        MAG_CK(cudaStreamSynchronize(stream));
        for (int w = 0; w < nw; ++w) {
            Tracked& T = tracked[which[w]];
            if (!T.out) {
                T.out = std::make_shared<std::ofstream>(dir + "/" + S.prm.name + "_traj_" + std::to_string(T.slot) +
                                                        ".dat");
                if (!*T.out) throw Error(-1, "print_trace: cannot open a file in " + dir);
            }
            const uint32_t* r = rec.data() + (size_t)w * 6;
            if (r[0] == 0) continue;  // removed
            float v[3];
            std::memcpy(v, r + 3, sizeof v);
            *T.out << std::setprecision(10) << x0 + (double)r[1] * inv * dx << ' ' << z0 + (double)r[2] * inv * dz
                   << ' ' << v[0] << ' ' << v[2] << ' ' << v[1] << std::endl;
        }
    }
}

// Pic::dist_reset (src/pic.cpp:412-420)
void Sim::dist_reset()
{
    const size_t nn = (size_t)nx * nz;
    dist.resize(sp.size());
    for (auto& d : dist) {
        d.bins.alloc(kEnergyBins);
        d.bins.zero(stream);
        d.stats.alloc(4);
        d.stats.zero(stream);
        d.rho_sum.alloc(nn);
        d.rho_sum.zero(stream);
    }
    u_sum.alloc(nn);
    u_sum.zero(stream);
    nsampl = 0;
}

// Pic::dist_sample (src/pic.cpp:421-428): per species the energy histogram and
// rho added to rhoAverage (BaseSpecies::dist_sample, src/particles.cpp:385-392),
// the potential added to uAvg (Fields::u_sample, src/fields.cpp:11-15).  rho is
// the charge deposit of the particles' current positions.
void Sim::dist_sample()
{
    ensure_full_u();
    if (dist.size() != sp.size()) dist_reset();
    const size_t nn = (size_t)nx * nz;
    if (rho_scratch.n < nn) rho_scratch.alloc(nn);
    for (size_t s = 0; s < sp.size(); ++s) {
        SpeciesState& S = sp[s];
        if (S.n_slots == 0) continue;
        launches += launch_energy_hist(S.x.p, S.vx.p, S.vy.p, S.vz.p, S.n_slots, S.prm.mass, kQe, 0.0, S.E_max,
                                       kEnergyBins, dist[s].bins.p, dist[s].stats.p, stream);
        rho_scratch.zero(stream);
        PushArgs pa = push_args((int)s, false);
        pa.rho = rho_scratch.p;
        launches += launch_deposit(pa, stream);
        launches += launch_axpy_i64(dist[s].rho_sum.p, rho_scratch.p, S.prm.charge * std::ldexp(1.0, -2 * kDepositShift),
                                    (long long)nn, stream);
    }
    launches += launch_axpy_f64(u_sum.p, u64.p, 1.0, (long long)nn, stream);
    ++nsampl;
    MAG_CK(cudaGetLastError());
}

void Sim::energy_dist(int s, std::vector<double>& pos, std::vector<double>& val, double stats[4])
{
    if (dist.size() != sp.size()) dist_reset();
    std::vector<unsigned long long> b(kEnergyBins);
    dist[s].bins.download(b.data(), kEnergyBins, stream);
    dist[s].stats.download(stats, 4, stream);
    MAG_CK(cudaStreamSynchronize(stream));
    const double mn = 0.0, mx = sp[s].E_max;
    const double norm = stats[0] * (mx - mn) / kEnergyBins;  // Histogram::norm
    pos.resize(kEnergyBins);
    val.resize(kEnergyBins);
    for (int i = 0; i < kEnergyBins; ++i) {
        pos[i] = mn + (mx - mn) * (i + .5) / kEnergyBins;  // Histogram::position
        val[i] = (double)b[i] / norm;
    }
}

void Sim::average(int which, double* out)
{
    if (dist.size() != sp.size()) dist_reset();
    const size_t nn = (size_t)nx * nz;
    std::vector<double> h(nn);
    if (which == 0) u_sum.download(h.data(), nn, stream);
    else if (which >= 5 && which - 5 < (int)sp.size()) dist[which - 5].rho_sum.download(h.data(), nn, stream);
    else throw Error(-1, "average: field must be MAG_U or MAG_SPECIES_RHO + species");
    MAG_CK(cudaStreamSynchronize(stream));
    const double f = 1.0 / nsampl;  // the reference's print factor 1.0/nsampl
    for (size_t k = 0; k < nn; ++k) out[k] = h[k] * f;
}

namespace {
// Field2D::print (src/Field2D.cpp:30-38): x, z, value per line, a blank line per x row
void print_field2d(const std::string& path, int nx, int nz, double dx, double dz, double x0, double z0,
                   const std::vector<double>& v)
{
    std::ofstream out(path);
    if (!out) throw Error(-6, "cannot open " + path + " for writing");
    for (int j = 0; j < nx; j++) {
        for (int l = 0; l < nz; l++) out << j * dx + x0 << "\t" << l * dz + z0 << "\t" << v[(size_t)j * nz + l] << std::endl;
        out << std::endl;
    }
}
}  // namespace

// Pic::print_distribution (src/pic.cpp:450-455) -> BaseSpecies::print_distribution
// (src/particles.cpp:376-383): <name>_energy_dist.dat and <name>_rho.dat
void Sim::print_distribution(const std::string& dir)
{
    const size_t nn = (size_t)nx * nz;
    for (size_t s = 0; s < sp.size(); ++s) {
        std::vector<double> pos, val;
        double st[4];
        energy_dist((int)s, pos, val, st);
        std::ofstream out(dir + "/" + species_prm[s].name + "_energy_dist.dat");
        if (!out) throw Error(-6, "cannot open " + dir + "/" + species_prm[s].name + "_energy_dist.dat");
        for (int i = 0; i < kEnergyBins; ++i) out << pos[i] << "\t" << val[i] << std::endl;  // Histogram::print
        std::vector<double> r(nn);
        average((int)(5 + s), r.data());
        print_field2d(dir + "/" + species_prm[s].name + "_rho.dat", nx, nz, dx, dz, x0, z0, r);
    }
}

// Pic::print_field (src/pic.cpp:456-459) -> Fields::u_print: uAvg / nsampl
void Sim::print_field(const std::string& path)
{
    std::vector<double> u((size_t)nx * nz);
    average(0, u.data());
    print_field2d(path, nx, nz, dx, dz, x0, z0, u);
}

// BaseSpecies::save (src/particles.cpp:32-57): the live particles as 64-byte
// t_particle records after the slot and live counts
void Sim::save_species(int s, const std::string& path)
{
    const int64_t n = sp[s].n_slots;
    ParticleFile f;
    for (auto* v : {&f.x, &f.z, &f.vx, &f.vy, &f.vz}) v->resize(n);
    int64_t m = 0;
    get_particles(s, n, f.x.data(), f.z.data(), f.vx.data(), f.vy.data(), f.vz.data(), nullptr, &m);
    for (auto* v : {&f.x, &f.z, &f.vx, &f.vy, &f.vz}) v->resize(m);
    f.y.assign(m, 0.0);
    f.ttd.assign(m, 0.0);
    if (multicoll && n) {  // time_to_death of the live particles, in slot order
        std::vector<double> t(n);
        std::vector<uint32_t> hx(n);
        sp[s].ttd.download(t.data(), n, stream);
        sp[s].x.download(hx.data(), n, stream);
        MAG_CK(cudaStreamSynchronize(stream));
        int64_t q = 0;
        for (int64_t k = 0; k < n && q < m; ++k)
            if (hx[k] != kDead) f.ttd[q++] = t[k];
    }
    f.total = (int32_t)std::max<int64_t>(n, m);
    write_particle_file(path, f);
}

// BaseSpecies::load (src/particles.cpp:59-93): the file's particles replace
// the species'; a position outside [x_min, x_max] or [z_min, z_max] is redrawn
// uniformly in that range, as the reference does for particles that left the
// domain in a non-self-consistent run
void Sim::load_species(int s, const std::string& path)
{
    ParticleFile f = read_particle_file(path);
    uint64_t st = seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(s + 1));
    auto uni = [&]() {  // SplitMix64 (Steele, Lea, Flood 2014) -> [0, 1)
        uint64_t z = (st += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (size_t i = 0; i < f.x.size(); ++i) {
        if (f.x[i] < x0 || f.x[i] > xmax) f.x[i] = (xmax - x0) * uni() + x0;
        if (f.z[i] < z0 || f.z[i] > zmax) f.z[i] = (zmax - z0) * uni() + z0;
    }
    set_particles(s, (int64_t)f.x.size(), f.x.data(), f.z.data(), f.vx.data(), f.vy.data(), f.vz.data());
    if (multicoll && !f.ttd.empty()) {  // the file's time_to_death replaces the drawn one
        sp[s].ttd.upload(f.ttd.data(), f.ttd.size(), stream);
        MAG_CK(cudaStreamSynchronize(stream));
    }
}

void Sim::set_rho_fixed(int s, const int64_t* in)
{
    MAG_CK(cudaStreamSynchronize(stream));
    sp[s].rho.upload((const unsigned long long*)in, (size_t)nx * nz, stream);
    MAG_CK(cudaStreamSynchronize(stream));
}

void Sim::get_rho_fixed(int s, int64_t* out)
{
    MAG_CK(cudaStreamSynchronize(stream));
    sp[s].rho.download((unsigned long long*)out, (size_t)nx * nz, stream);
    MAG_CK(cudaStreamSynchronize(stream));
}

Counters Sim::counters(int s)
{
    Counters c{};
    MAG_CK(cudaStreamSynchronize(stream));
    MAG_CK(cudaMemcpy(&c, sp[s].cnt.p, sizeof c, cudaMemcpyDeviceToHost));
    // the last launch's per-step counts are folded by the next launch only
    if (sp[s].launches > 0) c.live_sum += c.live_par[(sp[s].launches - 1) & 1];
    return c;
}

uint64_t Sim::niter(int s) { return sp[s].niter; }

void Sim::energy(int s, double& sum_v2, unsigned long long& n)
{
    Counters c;
    const int e = diag(s, sum_v2, n, c);
    if (e != 0) throw Error(e, "device error " + std::to_string(e));
}

// Sum of v^2 and count of the live particles with the species' counters and
// the device status (returned): one reduction kernel, one gather into
// page-locked host memory, one synchronisation
int Sim::diag(int s, double& sum_v2, unsigned long long& n, Counters& c)
{
    if (!diag_dev.p) diag_dev.alloc(2);
    SpeciesState& S = sp[s];
    MAG_CK(cudaMemsetAsync(diag_dev.p, 0, 2 * sizeof(double), stream));
    launches += launch_energy(S.x.p, S.vx.p, S.vy.p, S.vz.p, S.n_slots, diag_dev.p,
                              reinterpret_cast<unsigned long long*>(diag_dev.p + 1), stream);
    const int err = gather_status(diag_dev.p);
    sum_v2 = status_host->sum_v2;
    n = status_host->n_live;
    c = status_host->c[s];
    // the last launch's per-step counts are folded by the next launch only
    if (S.launches > 0) c.live_sum += c.live_par[(S.launches - 1) & 1];
    return err;
}

// New voltages of the electrodes (t_grid::voltage on its FIXED and FIXED_RF
// nodes; the free nodes' entries are ignored): the RF Laplace solution and,
// without a self-consistent field, the static potential are solved again as
// the Pic constructor does (pic.cpp:170-186); a self-consistent run's next
// step solves with them (the stored electrode potential of the direct solve
// is recomputed).
void Sim::set_voltages(const double* v, size_t n)
{
    if (n != (size_t)nx * nz) throw Error(-1, "electrode voltages: one value per node expected");
    if (p.electric_field_from_file) throw Error(-1, "electrode voltages: the fields come from files");
    for (size_t k = 0; k < n; ++k)
        if (mask[k] == 0 || mask[k] == 1) voltage[k] = v[k];
    MAG_CK(cudaStreamSynchronize(stream));
    d_volt.upload(voltage.data(), n, stream);
    if (u_prev_valid.p) u_prev_valid.zero(stream);
    ensure_full_u();
    setup_solver();
    solve(true, 0, false, false);
    if (!p.selfconsistent) solve(false, 0, false, false);
    refresh_rf_pairs();
    if (green_ready()) {  // the potential of the electrodes alone
        SolveArgs vac = solve_args(false, 0, false);
        vac.u = green_vac.p;
        vac.Exf = nullptr;
        vac.Ezf = nullptr;
        vac.status = green_status.p;
        GreenArgs g = green_args(false);
        g.rows = nullptr;
        launches += launch_green_solve(vac, g, stream);
    }
    MAG_CK(cudaGetLastError());
}

// ---- particle source --------------------------------------------------

SourceArgs Sim::source_args(int s, bool init)
{
    SpeciesState& S = sp[s];
    SourceState& Q = src[s];
    SourceArgs a{};
    a.x = Q.x.p;
    a.z = Q.z.p;
    a.vx = Q.vx.p;
    a.vy = Q.vy.p;
    a.vz = Q.vz.p;
    a.n = Q.n;
    a.count = Q.count.p;
    a.rec = Q.rec.p;
    a.dropped = Q.dropped.p;
    a.cnt = S.cnt.p;
    a.lx = xmax - x0;
    a.lz = zmax - z0;
    a.factor = std::max(Q.factor, 1);
    a.bx = a.lx / a.factor;
    a.bz = a.lz / a.factor;
    a.dt = S.prm.dt;
    const PushArgs pa = push_args(s, init);
    a.hq = pa.hq;
    a.ez = pa.extern_ez;
    a.tx = pa.tx;
    a.ty = pa.ty;
    a.tz = pa.tz;
    a.sx = pa.sx;
    a.sy = pa.sy;
    a.sz = pa.sz;
    a.prob = (float)S.prob;
    a.coll = !init && coll_mode(s) != 0 ? 1 : 0;
    a.species = (uint32_t)s;
    a.seed = seed;
    a.step = S.niter;
    return a;
}

// Species<CARTESIAN>::source5_refresh (src/particles.cpp:1052-1082) for every
// species that holds particles: N / factor box particles, N = density V.
void Sim::source_refresh(int factor)
{
    if (factor < 1) throw Error(-1, "source refresh: factor must be >= 1");
    if (p.coord != CARTESIAN) throw Error(-1, "use_source: Species<CYLINDRICAL>::source is not defined in the reference");
    src.resize(sp.size());
    for (size_t s = 0; s < sp.size(); ++s) {
        SpeciesState& S = sp[s];
        SourceState& Q = src[s];
        Q.factor = factor;
        if (S.n_slots == 0) continue;  // "checks if we simulate this species as particles"
        if (coll_mode((int)s) != 0 && any_target_slots((int)s))
            throw Error(-1, "use_source: source box collisions with particle partners are not provided by this library");
        const int64_t n = (int64_t)(unsigned)(S.prm.density * p.V / factor);
        Q.n = n;
        for (auto* a : {&Q.x, &Q.z}) a->alloc(std::max<int64_t>(n, 1));
        for (auto* a : {&Q.vx, &Q.vy, &Q.vz}) a->alloc(std::max<int64_t>(n, 1));
        Q.count.alloc(std::max<int64_t>(n, 1));
        Q.offs.alloc(std::max<int64_t>(n, 1));
        Q.rec.alloc((size_t)std::max<int64_t>(n, 1) * kMaxInject * 5);
        Q.total.alloc(1);
        Q.dropped.alloc(1);
        Q.dropped.zero(stream);
        launches += launch_source_refresh(source_args((int)s, true), (float)(S.v_max / std::sqrt(2.0)), stream);
    }
    MAG_CK(cudaStreamSynchronize(stream));
}

// Species<CARTESIAN>::source (src/particles.cpp:1165-1226) after the species'
// push: the box step, then its copies appended to the species (the count is
// read back to size the arrays).
void Sim::source_step(int s)
{
    SourceState& Q = src[s];
    if (Q.n == 0) return;
    SpeciesState& S = sp[s];
    const SourceArgs a = source_args(s, false);
    const CollideArgs c = a.coll ? collide_args(s) : CollideArgs{};
    launches += launch_source_step(a, c, Q.offs.p, Q.total.p, stream);
    long long total = 0;
    MAG_CK(cudaMemcpyAsync(&total, Q.total.p, sizeof total, cudaMemcpyDeviceToHost, stream));
    MAG_CK(cudaStreamSynchronize(stream));
    if (total <= 0) return;
    ensure_capacity(s, S.n_slots + total);
    SourceAppend t{};
    t.x = S.x.p;
    t.z = S.z.p;
    t.vx = S.vx.p;
    t.vy = S.vy.p;
    t.vz = S.vz.p;
    t.id = S.id.p;
    t.rho = p.selfconsistent ? S.rho.p : nullptr;
    t.base = S.n_slots;
    t.next_id = S.next_id;
    t.nx = nx;
    t.nz = nz;
    t.dx = dx;
    t.dz = dz;
    launches += launch_source_append(a, Q.offs.p, t, stream);
    S.n_slots += total;
    S.next_id += (uint32_t)total;
    Q.injected += (uint64_t)total;
    upload_slots(s);
}

// BaseSpecies::source5_save (src/particles.cpp:109-120)
void Sim::source_save(int s, const std::string& path)
{
    SourceState& Q = src[s];
    ParticleFile f;
    const int64_t n = Q.n;
    for (auto* v : {&f.x, &f.z, &f.vx, &f.vy, &f.vz}) v->resize(n);
    std::vector<float> v3[3];
    for (auto& v : v3) v.resize(n);
    if (n) {
        Q.x.download(f.x.data(), n, stream);
        Q.z.download(f.z.data(), n, stream);
        Q.vx.download(v3[0].data(), n, stream);
        Q.vy.download(v3[1].data(), n, stream);
        Q.vz.download(v3[2].data(), n, stream);
    }
    MAG_CK(cudaStreamSynchronize(stream));
    for (int64_t i = 0; i < n; ++i) {
        f.vx[i] = v3[0][i];
        f.vy[i] = v3[1][i];
        f.vz[i] = v3[2][i];
    }
    write_source_file(path, f);
}

// BaseSpecies::source5_load (src/particles.cpp:122-140): false (and the box
// unchanged) when the file cannot be opened, as the reference only warns
bool Sim::source_load(int s, const std::string& path)
{
    ParticleFile f;
    if (!read_source_file(path, f)) return false;
    SourceState& Q = src[s];
    const int64_t n = (int64_t)f.x.size();
    if (Q.factor == 0) Q.factor = std::max(p.src_fact, 1);
    Q.n = n;
    for (auto* a : {&Q.x, &Q.z}) a->alloc(std::max<int64_t>(n, 1));
    for (auto* a : {&Q.vx, &Q.vy, &Q.vz}) a->alloc(std::max<int64_t>(n, 1));
    Q.count.alloc(std::max<int64_t>(n, 1));
    Q.offs.alloc(std::max<int64_t>(n, 1));
    Q.rec.alloc((size_t)std::max<int64_t>(n, 1) * kMaxInject * 5);
    Q.total.alloc(1);
    Q.dropped.alloc(1);
    Q.dropped.zero(stream);
    std::vector<float> v3[3];
    for (auto& v : v3) v.resize(n);
    for (int64_t i = 0; i < n; ++i) {
        v3[0][i] = (float)f.vx[i];
        v3[1][i] = (float)f.vy[i];
        v3[2][i] = (float)f.vz[i];
    }
    Q.x.upload(f.x.data(), n, stream);
    Q.z.upload(f.z.data(), n, stream);
    Q.vx.upload(v3[0].data(), n, stream);
    Q.vy.upload(v3[1].data(), n, stream);
    Q.vz.upload(v3[2].data(), n, stream);
    MAG_CK(cudaStreamSynchronize(stream));
    return true;
}

}  // namespace mag
