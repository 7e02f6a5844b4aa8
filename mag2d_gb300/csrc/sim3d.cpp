// The 3D Cartesian run on the GPU (sim3d.hpp).
#include "sim3d.hpp"

#include <algorithm>
#include <cmath>

#include "kernels.hpp"

namespace mag {

Sim3D::Sim3D(const std::string& config, const std::string& species_conf, const SimOptions& opts)
{
    device = opts.device;
    seed = opts.seed ? opts.seed : 1;
    if (opts.poisson_tol > 0) tol = opts.poisson_tol;
    if (opts.poisson_max_iter > 0) max_iter = opts.poisson_max_iter;
    p = make_param(KeyValueConfig::from_file(config));
    if (p.coord != CARTESIAN3D) throw Error(-1, "the 3D handle needs coord = CARTESIAN3D");
    if (p.mover != ADVANCE_BORIS) throw Error(-1, "CARTESIAN3D: only ADVANCE_BORIS (Species<CARTESIAN3D>::advance)");
    if (!p.magnetic_field_const) throw Error(-1, "CARTESIAN3D: magnetic field tables are not provided (constant B)");
    if (p.use_source) throw Error(-1, "CARTESIAN3D: particle sources are not defined for the 3D species");
    parse_species_conf(species_conf, species_prm, inters);
    if (species_prm.empty()) throw Error(-1, "species_conf defines no species");
    if ((int)species_prm.size() > kMaxSpecies) throw Error(-1, "too many species");
    if ((int)inters.size() > kMaxInteractions) throw Error(-1, "too many interactions");
    nx = p.x_sampl;
    ny = p.y_sampl;
    nz = p.z_sampl;
    if (nx < 3 || ny < 3 || nz < 3 || nx > 4096 || ny > 4096 || nz > 4096)
        throw Error(-1, "CARTESIAN3D: every axis needs 3..4096 nodes");
    dx = p.dx;
    dy = p.dy;
    dz = p.dz;
    xmax = p.x_max;
    ymax = p.y_max;
    zmax = p.z_max;
    const size_t nn = (size_t)nx * ny * nz;
    // Geometry::Geometry (fields3d.cpp:11-31): the box faces fixed at 0 V and
    // the Quadrupole placeholder electrode (one node at the centre, 1 V)
    mask.assign(nn, 0);
    voltage.assign(nn, 0.0);
    for (int i = 0; i < nx; ++i)
        for (int j = 0; j < ny; ++j)
            for (int k = 0; k < nz; ++k)
                if (i == 0 || i == nx - 1 || j == 0 || j == ny - 1 || k == 0 || k == nz - 1)
                    mask[((size_t)i * ny + j) * nz + k] = 1;
    const size_t c = ((size_t)(nx / 2) * ny + ny / 2) * nz + nz / 2;
    mask[c] = 1;
    voltage[c] = 1.0;
    std::vector<uint8_t> cellfree((size_t)(nx - 1) * (ny - 1) * (nz - 1));
    for (int i = 0; i < nx - 1; ++i)
        for (int j = 0; j < ny - 1; ++j)
            for (int k = 0; k < nz - 1; ++k) {
                bool f = false;
                for (int q = 0; q < 8; ++q)
                    f = f || mask[((size_t)(i + (q & 1)) * ny + j + ((q >> 1) & 1)) * nz + k + (q >> 2)] == 0;
                cellfree[((size_t)i * (ny - 1) + j) * (nz - 1) + k] = f ? 1 : 0;
            }
    MAG_CK(cudaSetDevice(device));
    if (opts.stream) {
        stream = opts.stream;
        own_stream = false;
    } else {
        MAG_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    }
    cudaDeviceProp prop{};
    MAG_CK(cudaGetDeviceProperties(&prop, device));
    sm_count = prop.multiProcessorCount;
    solve_blocks = std::max(1, std::min<int>(solve3d_blocks(sm_count), (int)((nn + 255) / 256)));
    d_mask.upload(mask.data(), nn, stream);
    d_volt.upload(voltage.data(), nn, stream);
    d_cellfree.upload(cellfree.data(), cellfree.size(), stream);
    for (auto* a : {&u, &b, &r, &pv, &qv}) {
        a->alloc(nn);
        a->zero(stream);
    }
    part.alloc((size_t)6 * solve_blocks);
    bar.alloc(2);
    bar.zero(stream);
    d_err.alloc(1);
    d_err.zero(stream);
    d_status.alloc(1);
    d_status.zero(stream);
    Exf.alloc((size_t)(nx + 1) * ny * nz);
    Eyf.alloc((size_t)nx * (ny + 1) * nz);
    Ezf.alloc((size_t)nx * ny * (nz + 1));
    e_sum.alloc(1);
    e_cnt.alloc(1);
    build_species(species_prm, inters, nn, stream, sp, d_inter, d_tables);
    ys.resize(sp.size());
    if (opts.capacity_hint > 0)
        for (size_t s = 0; s < sp.size(); ++s) ensure_capacity((int)s, opts.capacity_hint);
    launches += launch_faces3d(u.p, nx, ny, nz, dx, dy, dz, Exf.p, Eyf.p, Ezf.p, stream);
    MAG_CK(cudaStreamSynchronize(stream));
}

Sim3D::~Sim3D()
{
    if (stream) {
        cudaSetDevice(device);
        cudaStreamSynchronize(stream);
        if (own_stream) cudaStreamDestroy(stream);
    }
}

int Sim3D::sync()
{
    MAG_CK(cudaStreamSynchronize(stream));
    int err = 0;
    MAG_CK(cudaMemcpy(&err, d_err.p, sizeof(int), cudaMemcpyDeviceToHost));
    MAG_CK(cudaMemcpy(&last_solve, d_status.p, sizeof(SolveStatus), cudaMemcpyDeviceToHost));
    for (auto& s : sp) {
        Counters c;
        MAG_CK(cudaMemcpy(&c, s.cnt.p, sizeof c, cudaMemcpyDeviceToHost));
        if (c.error && !err) err = c.error;
    }
    if (err) {
        int zero = 0;
        MAG_CK(cudaMemcpy(d_err.p, &zero, sizeof(int), cudaMemcpyHostToDevice));
    }
    return err;
}

void Sim3D::ensure_capacity(int s, int64_t need)
{
    SpeciesState& S = sp[s];
    if (need <= S.cap) return;
    int64_t cap = std::max<int64_t>(need, (int64_t)(S.cap * 1.5) + 1024);
    cap = (cap + kSlotAlign - 1) / kSlotAlign * kSlotAlign;
    MAG_CK(cudaStreamSynchronize(stream));
    auto grow = [&](auto& a) {
        typename std::remove_reference<decltype(a)>::type nb;
        nb.alloc(cap);
        if (S.n_slots)
            MAG_CK(cudaMemcpyAsync(nb.p, a.p, S.n_slots * sizeof(*a.p), cudaMemcpyDeviceToDevice, stream));
        MAG_CK(cudaStreamSynchronize(stream));
        a = std::move(nb);
    };
    grow(S.x);
    grow(ys[s]);
    grow(S.z);
    grow(S.vx);
    grow(S.vy);
    grow(S.vz);
    grow(S.id);
    S.cand.alloc(cap);
    S.cand_rec.alloc(cap);
    S.cap = cap;
}

void Sim3D::upload_slots(int s)
{
    const unsigned long long v = (unsigned long long)sp[s].n_slots;
    MAG_CK(cudaMemcpyAsync(&sp[s].cnt.p->slots, &v, sizeof v, cudaMemcpyHostToDevice, stream));
    MAG_CK(cudaStreamSynchronize(stream));
}

// the species' particles replaced by n particles (positions in [0, max] per
// axis, others removed), converted to the fixed-point SoA on the device
void Sim3D::set_particles(int s, int64_t n, const double* x, const double* y, const double* z, const double* vx,
                          const double* vy, const double* vz)
{
    SpeciesState& S = sp[s];
    S.n_slots = 0;
    ensure_capacity(s, std::max<int64_t>(n, 1));
    if (stage.n < (size_t)(6 * n)) stage.alloc((size_t)(6 * n));
    const double* src[6] = {x, y, z, vx, vy, vz};
    for (int c = 0; c < 6; ++c)
        if (n)
            MAG_CK(cudaMemcpyAsync(stage.p + (size_t)c * n, src[c], (size_t)n * sizeof(double), cudaMemcpyHostToDevice,
                                   stream));
    const Set3Geom g{xmax, ymax, zmax, dx, dy, dz};
    launches += launch_set_particles3d(stage.p, n, g, S.x.p, ys[s].p, S.z.p, S.vx.p, S.vy.p, S.vz.p, S.id.p, stream);
    S.n_slots = n;
    S.next_id = (uint32_t)n;
    upload_slots(s);
}

void Sim3D::get_particles(int s, int64_t cap, double* x, double* y, double* z, double* vx, double* vy, double* vz,
                          uint32_t* id, int64_t* n_out)
{
    SpeciesState& S = sp[s];
    const int64_t n = S.n_slots;
    std::vector<uint32_t> hx(n), hy(n), hz(n), hid(n);
    std::vector<float> hvx(n), hvy(n), hvz(n);
    S.x.download(hx.data(), n, stream);
    ys[s].download(hy.data(), n, stream);
    S.z.download(hz.data(), n, stream);
    S.vx.download(hvx.data(), n, stream);
    S.vy.download(hvy.data(), n, stream);
    S.vz.download(hvz.data(), n, stream);
    S.id.download(hid.data(), n, stream);
    MAG_CK(cudaStreamSynchronize(stream));
    const double inv = 1.0 / (double)(1u << kFracBits);
    int64_t m = 0;
    for (int64_t k = 0; k < n && m < cap; ++k) {
        if (hx[k] == kDead) continue;
        if (x) x[m] = (double)hx[k] * inv * dx;
        if (y) y[m] = (double)hy[k] * inv * dy;
        if (z) z[m] = (double)hz[k] * inv * dz;
        if (vx) vx[m] = hvx[k];
        if (vy) vy[m] = hvy[k];
        if (vz) vz[m] = hvz[k];
        if (id) id[m] = hid[k];
        ++m;
    }
    *n_out = m;
}

Push3Args Sim3D::push_args(int s, bool init)
{
    SpeciesState& S = sp[s];
    Push3Args a{};
    a.x = S.x.p;
    a.y = ys[s].p;
    a.z = S.z.p;
    a.vx = S.vx.p;
    a.vy = S.vy.p;
    a.vz = S.vz.p;
    a.id = S.id.p;
    a.n = S.n_slots;
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    const double one = (double)(1u << kFracBits);
    a.xmaxf = (uint32_t)std::llrint((nx - 1) * one);
    a.ymaxf = (uint32_t)std::llrint((ny - 1) * one);
    a.zmaxf = (uint32_t)std::llrint((nz - 1) * one);
    a.periodic = p.boundary == BND_PERIODIC ? 1 : 0;
    a.init = init ? 1 : 0;
    a.cellfree = d_cellfree.p;
    a.Exf = Exf.p;
    a.Eyf = Eyf.p;
    a.Ezf = Ezf.p;
    const double q = S.prm.charge, m = S.prm.mass, dt = S.prm.dt;
    const double rot = init ? -0.5 * q * dt / (2.0 * m) : q * dt / (2.0 * m);
    a.hq = (float)(init ? -q / m * dt / 2.0 : q / m * dt / 2.0);
    // (Br, Bt, Bz) of the config as (Bx, By, Bz)
    const double tx = p.Br * rot, ty = p.Bt * rot, tz = p.Bz * rot;
    const double f = 2.0 / (1 + tx * tx + ty * ty + tz * tz);
    a.tx = (float)tx;
    a.ty = (float)ty;
    a.tz = (float)tz;
    a.sx = (float)(tx * f);
    a.sy = (float)(ty * f);
    a.sz = (float)(tz * f);
    a.has_b = (p.Br != 0.0 || p.Bt != 0.0 || p.Bz != 0.0) ? 1 : 0;
    a.cx = (float)(dt / dx);
    a.cy = (float)(dt / dy);
    a.cz = (float)(dt / dz);
    a.rho = p.selfconsistent && !init ? S.rho.p : nullptr;
    a.coll_threshold = init ? 0u : S.threshold;
    a.species = (uint32_t)s;
    a.seed = seed;
    a.step = S.niter;
    a.cand = S.cand.p;
    a.cand_rec = S.cand_rec.p;
    a.cnt = S.cnt.p;
    a.slot = (int)(S.launches & 1);
    a.fold_slot = S.launches > 0 ? (int)((S.launches - 1) & 1) : -1;
    return a;
}

CollideArgs Sim3D::collide_args(int s)
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
    bool any = false;
    for (size_t t = 0; t < sp.size(); ++t) {
        a.t_has_slots[t] = sp[t].n_slots > 0 ? 1 : 0;
        a.t_x[t] = sp[t].x.p;
        a.t_vx[t] = sp[t].vx.p;
        a.t_vy[t] = sp[t].vy.p;
        a.t_vz[t] = sp[t].vz.p;
        a.t_n[t] = sp[t].n_slots;
        any = any || (t < S.rates.size() && S.rates[t] > 0.0 && sp[t].n_slots > 0);
    }
    a.any_target_slots = any ? 1 : 0;
    a.seed = seed;
    a.species = (uint32_t)s;
    a.step = S.niter;
    a.slot = (int)(S.launches & 1);
    return a;
}

void Sim3D::run_solve(bool from_rho64, bool clear_rho)
{
    Solve3Args a{};
    a.nx = nx;
    a.ny = ny;
    a.nz = nz;
    a.nsp = (int)sp.size();
    a.mask = d_mask.p;
    a.voltage = d_volt.p;
    a.u = u.p;
    a.b = b.p;
    a.r = r.p;
    a.p = pv.p;
    a.qv = qv.p;
    a.part = part.p;
    for (size_t s = 0; s < sp.size(); ++s) {
        a.rho_fixed[s] = sp[s].rho.p;
        a.rho_weight[s] = sp[s].prm.charge * std::ldexp(1.0, -3 * kDeposit3Bits);
    }
    a.rho64 = from_rho64 ? rho64.p : nullptr;
    a.rho_scale = from_rho64 ? 1.0 / kEps0 : p.macroparticle_factor / (dx * dy * dz * kEps0);
    a.ix2 = 1.0 / (dx * dx);
    a.iy2 = 1.0 / (dy * dy);
    a.iz2 = 1.0 / (dz * dz);
    a.tol = tol;
    a.max_iter = max_iter;
    a.clear_rho = clear_rho ? 1 : 0;
    a.bar = bar.p;
    a.err = d_err.p;
    a.status = d_status.p;
    launches += launch_solve3d(a, solve_blocks, stream);
    launches += launch_faces3d(u.p, nx, ny, nz, dx, dy, dz, Exf.p, Eyf.p, Ezf.p, stream);
    MAG_CK(cudaGetLastError());
}

// ElMag3D::solve (fields3d.cpp:78-90) of a given charge density, or of the
// species deposits (left in place)
SolveStatus Sim3D::solve(const double* rho_host)
{
    const size_t nn = (size_t)nx * ny * nz;
    if (rho_host) {
        if (rho64.n < nn) rho64.alloc(nn);
        rho64.upload(rho_host, nn, stream);
    }
    run_solve(rho_host != nullptr, false);
    const int e = sync();
    if (e) throw Error(e, "3D Poisson solve failed (device status " + std::to_string(e) + ")");
    return last_solve;
}

// the field of the start (self-consistent: from the particles' deposit;
// otherwise the electrode alone), then the leapfrog start of every species
void Sim3D::advance_init()
{
    MAG_CK(cudaSetDevice(device));
    for (size_t s = 0; s < sp.size(); ++s) {
        sp[s].rho.zero(stream);
        if (p.selfconsistent && sp[s].n_slots > 0) {
            Push3Args a = push_args((int)s, false);
            a.rho = sp[s].rho.p;
            launches += launch_deposit3d(a, stream);
        }
    }
    run_solve(false, true);
    for (size_t s = 0; s < sp.size(); ++s) {
        if (sp[s].n_slots == 0) continue;
        launches += launch_push3d(push_args((int)s, true), sm_count, stream);
    }
    MAG_CK(cudaGetLastError());
}

void Sim3D::step()
{
    if (p.selfconsistent) run_solve(false, true);
    for (size_t s = 0; s < sp.size(); ++s) {
        SpeciesState& S = sp[s];
        if (S.n_slots == 0) {
            S.niter++;
            continue;
        }
        const Push3Args a = push_args((int)s, false);
        launches += launch_push3d(a, sm_count, stream);
        if (S.threshold != 0u) {
            const CollideArgs ca = collide_args((int)s);
            const double expect = (double)S.n_slots * S.prob;
            const int grid = (int)std::min<double>(4.0 * sm_count, std::ceil(4.0 * expect / 128.0) + 1.0);
            launches += launch_collide(ca, grid, stream);
        }
        S.launches++;
        S.niter++;
    }
}

void Sim3D::advance(uint64_t nsteps)
{
    MAG_CK(cudaSetDevice(device));
    for (uint64_t k = 0; k < nsteps; ++k) step();
    MAG_CK(cudaGetLastError());
}

void Sim3D::get_field(int which, double* out)
{
    const size_t nn = (size_t)nx * ny * nz;
    MAG_CK(cudaStreamSynchronize(stream));
    if (which == 0) {
        u.download(out, nn, stream);
        MAG_CK(cudaStreamSynchronize(stream));
    } else if (which == 3) {
        // the reference's codes: FIXED 0 on the box faces, the electrode's id
        // -1 at the centre, FREE 2
        const size_t c = ((size_t)(nx / 2) * ny + ny / 2) * nz + nz / 2;
        for (size_t k = 0; k < nn; ++k) out[k] = mask[k] ? (k == c ? -1.0 : 0.0) : 2.0;
    } else if (which == 2) {
        // charge per node [C] as Field3D::accumulate(charge, ...) sums it
        std::fill(out, out + nn, 0.0);
        std::vector<int64_t> acc(nn);
        for (size_t s = 0; s < sp.size(); ++s) {
            get_rho_fixed((int)s, acc.data());
            const double w = sp[s].prm.charge * std::ldexp(1.0, -3 * kDeposit3Bits);
            for (size_t k = 0; k < nn; ++k) out[k] += w * (double)(uint64_t)acc[k];
        }
    } else {
        throw Error(-1, "3D field: MAG_U, MAG_RHO or MAG_MASK");
    }
}

void Sim3D::get_rho_fixed(int s, int64_t* out)
{
    MAG_CK(cudaStreamSynchronize(stream));
    sp[s].rho.download((unsigned long long*)out, (size_t)nx * ny * nz, stream);
    MAG_CK(cudaStreamSynchronize(stream));
}

Counters Sim3D::counters(int s)
{
    Counters c{};
    MAG_CK(cudaStreamSynchronize(stream));
    MAG_CK(cudaMemcpy(&c, sp[s].cnt.p, sizeof c, cudaMemcpyDeviceToHost));
    if (sp[s].launches > 0) c.live_sum += c.live_par[(sp[s].launches - 1) & 1];
    return c;
}

void Sim3D::energy(int s, double& sum_v2, unsigned long long& n)
{
    e_sum.zero(stream);
    e_cnt.zero(stream);
    SpeciesState& S = sp[s];
    launches += launch_energy(S.x.p, S.vx.p, S.vy.p, S.vz.p, S.n_slots, e_sum.p, e_cnt.p, stream);
    MAG_CK(cudaStreamSynchronize(stream));
    sum_v2 = 0;
    n = 0;
    if (S.n_slots) {
        MAG_CK(cudaMemcpy(&sum_v2, e_sum.p, 8, cudaMemcpyDeviceToHost));
        MAG_CK(cudaMemcpy(&n, e_cnt.p, 8, cudaMemcpyDeviceToHost));
    }
}

}  // namespace mag
