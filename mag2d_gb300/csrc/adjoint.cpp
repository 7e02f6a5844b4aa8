// Adjoint runs (adjoint.hpp).  Forward: the library's own step, with the
// particle state (and the potential, the solve's warm start) saved every K
// steps.  Backward, segment by segment from the end: restore the segment's
// checkpoint, recompute its K steps keeping each step's state and potential,
// then walk the steps in reverse:
//   particle adjoint (k_adj_push)  -> face adjoints, d/dB
//   faces -> node adjoints g        (transpose of the face differences)
//   transpose Poisson solve          A^-T g = W A^-1 W^-1 g, W = row weights that
//                                    make the reference's operator symmetric
//   Dirichlet nodes                  -> d/d(voltage keys) through the geometry basis
//   deposit adjoint                  -> position adjoints of the step's start
// and finally the leapfrog start and the potential it used.
#include "adjoint.hpp"

#include <algorithm>
#include <cmath>

#include "kernels.hpp"

namespace mag {

namespace {

constexpr double kPiA = 3.14159265358979323846;

struct Snap {
    DevArray<uint32_t> x, z;
    DevArray<float> vx, vy, vz;
    int64_t n = 0;
};

void take(Snap& d, const SpeciesState& S, cudaStream_t s)
{
    d.n = S.n_slots;
    if (d.x.n < (size_t)d.n) {
        d.x.alloc(d.n);
        d.z.alloc(d.n);
        d.vx.alloc(d.n);
        d.vy.alloc(d.n);
        d.vz.alloc(d.n);
    }
    if (!d.n) return;
    MAG_CK(cudaMemcpyAsync(d.x.p, S.x.p, d.n * 4, cudaMemcpyDeviceToDevice, s));
    MAG_CK(cudaMemcpyAsync(d.z.p, S.z.p, d.n * 4, cudaMemcpyDeviceToDevice, s));
    MAG_CK(cudaMemcpyAsync(d.vx.p, S.vx.p, d.n * 4, cudaMemcpyDeviceToDevice, s));
    MAG_CK(cudaMemcpyAsync(d.vy.p, S.vy.p, d.n * 4, cudaMemcpyDeviceToDevice, s));
    MAG_CK(cudaMemcpyAsync(d.vz.p, S.vz.p, d.n * 4, cudaMemcpyDeviceToDevice, s));
}

void give(const Snap& d, SpeciesState& S, cudaStream_t s)
{
    if (!d.n) return;
    MAG_CK(cudaMemcpyAsync(S.x.p, d.x.p, d.n * 4, cudaMemcpyDeviceToDevice, s));
    MAG_CK(cudaMemcpyAsync(S.z.p, d.z.p, d.n * 4, cudaMemcpyDeviceToDevice, s));
    MAG_CK(cudaMemcpyAsync(S.vx.p, d.vx.p, d.n * 4, cudaMemcpyDeviceToDevice, s));
    MAG_CK(cudaMemcpyAsync(S.vy.p, d.vy.p, d.n * 4, cudaMemcpyDeviceToDevice, s));
    MAG_CK(cudaMemcpyAsync(S.vz.p, d.vz.p, d.n * 4, cudaMemcpyDeviceToDevice, s));
}

void copy_d(DevArray<double>& dst, const DevArray<double>& src, size_t n, cudaStream_t s)
{
    if (dst.n < n) dst.alloc(n);
    MAG_CK(cudaMemcpyAsync(dst.p, src.p, n * 8, cudaMemcpyDeviceToDevice, s));
}

}  // namespace

AdjointResult Adjoint::run(Sim& sim, const AdjointConfig& cfg)
{
    MAG_CK(cudaSetDevice(sim.device));
    cudaStream_t st = sim.stream;
    if (cfg.nsteps == 0) throw Error(-1, "adjoint run: nsteps must be positive");
    if (!sim.p.magnetic_field_const) throw Error(-1, "adjoint run: a magnetic field table is not supported (constant B only)");
    if (sim.p.use_source) throw Error(-1, "adjoint run: particle sources (use_source) are not supported");
    if (sim.p.u_smooth) throw Error(-1, "adjoint run: potential smoothing (u_smooth) is not supported");
    // checkpoints copy and restore u: every solve of the run computes every node
    sim.ensure_full_u();
    // and every replayed step solves from the same start as the forward one
    struct RowsGuard {
        Sim& s;
        bool old_rows, old_extrapolate;
        ~RowsGuard()
        {
            s.partial_rows = old_rows;
            s.extrapolate_u = old_extrapolate;
        }
    } guard{sim, sim.partial_rows, sim.extrapolate_u};
    sim.partial_rows = false;
    sim.extrapolate_u = false;
    if (sim.emode == 2) throw Error(-1, "adjoint run: RF fields are not supported (static and self-consistent fields only)");
    for (auto& S : sim.sp)
        if (S.threshold != 0)
            throw Error(-1, "adjoint run: collisions must be off (the adjoint is of the collisionless step)");
    const bool sc = sim.p.selfconsistent != 0;
    const int nx = sim.nx, nz = sim.nz;
    const size_t nn = (size_t)nx * nz;
    const int coord = sim.p.coord == CYLINDRICAL ? 1 : 0;
    const uint64_t N = cfg.nsteps;
    const int K = std::max(1, cfg.checkpoint);
    const int nseg = (int)((N + K - 1) / K);
    const int np = (int)cfg.voltage_keys.size();
    const int nb = cfg.grad_b ? 3 : 0;
    sim.setup_solver();

    // geometry basis of each voltage key on the FIXED nodes: d voltage / d key
    std::vector<double> basis((size_t)np * nn, 0.0);
    {
        const KeyValueConfig base = KeyValueConfig::from_file(sim.config_path);
        for (int q = 0; q < np; ++q) {
            std::vector<int8_t> m0, m1;
            std::vector<double> v0, v1;
            KeyValueConfig c0 = base, c1 = base;
            c0.set(cfg.voltage_keys[q], "0");
            c1.set(cfg.voltage_keys[q], "1");
            build_geometry(make_param(c0), m0, v0);
            build_geometry(make_param(c1), m1, v1);
            if (v0.size() != nn) throw Error(-1, "adjoint run: geometry size mismatch");
            bool any = false;
            for (size_t k = 0; k < nn; ++k)
                if (sim.mask[k] == 0) {
                    basis[(size_t)q * nn + k] = v1[k] - v0[k];
                    any = any || v1[k] != v0[k];
                }
            if (!any) throw Error(-1, "adjoint run: key '" + cfg.voltage_keys[q] + "' sets no electrode voltage");
        }
    }
    // row weights W (symmetrise the operator) and the right-hand-side scaling of the solve
    std::vector<double> w(nx), scale(nx), wsc(nx);
    for (int i = 0; i < nx; ++i) {
        if (coord == 1) {
            w[i] = i > 0 ? (double)i : 0.125;
            scale[i] = i > 0 ? -1.0 / kEps0 / (kPiA * sim.dx * sim.dx * 2.0 * i * sim.dz) * sim.p.macroparticle_factor
                             : -1.0 / kEps0 / (kPiA * sim.dx * sim.dx * 0.25 * sim.dz) * sim.p.macroparticle_factor;
        } else {
            w[i] = 1.0;
            scale[i] = -(sim.dx * sim.dx) / kEps0 / sim.p.dV;
        }
        wsc[i] = w[i] * scale[i];
    }
    DevArray<double> d_basis, d_w, d_scale, d_wsc, d_grad, zeros, g, g_static, adj_rho, adj_u, y, lrho, u_init;
    d_basis.upload(basis.data(), basis.size(), st);
    d_w.upload(w.data(), w.size(), st);
    d_scale.upload(scale.data(), scale.size(), st);
    d_wsc.upload(wsc.data(), wsc.size(), st);
    d_grad.alloc(np + 3);
    d_grad.zero(st);
    for (auto* a : {&zeros, &g, &g_static, &adj_rho, &adj_u, &y, &lrho}) {
        a->alloc(nn);
        a->zero(st);
    }
    DevArray<float> lExf, lEzf, Exf_t, Ezf_t;
    lExf.alloc((size_t)(nx + 1) * nz);
    lEzf.alloc((size_t)nx * (nz + 1));
    Exf_t.alloc((size_t)(nx + 1) * nz);
    Ezf_t.alloc((size_t)nx * (nz + 1));

    const int ns = (int)sim.sp.size();
    const int saved_sort = sim.sort_interval;
    sim.sort_interval = -1;
    sim.sort_due = false;

    // ---- forward ---------------------------------------------------------
    std::vector<Snap> init_state(ns);
    for (int s = 0; s < ns; ++s) take(init_state[s], sim.sp[s], st);
    sim.advance_init();
    copy_d(u_init, sim.u64, nn, st);
    std::vector<std::vector<Snap>> ckpt(nseg);
    for (auto& c : ckpt) c.resize(ns);
    std::vector<DevArray<double>> ckpt_u(nseg);
    for (uint64_t n = 0; n < N; ++n) {
        if (n % (uint64_t)K == 0) {
            const int sg = (int)(n / K);
            for (int s = 0; s < ns; ++s) take(ckpt[sg][s], sim.sp[s], st);
            copy_d(ckpt_u[sg], sim.u64, nn, st);
        }
        sim.step();
    }
    std::vector<Snap> final_state(ns);
    for (int s = 0; s < ns; ++s) take(final_state[s], sim.sp[s], st);
    DevArray<double> final_u;
    copy_d(final_u, sim.u64, nn, st);
    std::vector<Counters> final_cnt(ns);
    std::vector<uint64_t> final_niter(ns), final_launches(ns);
    const uint64_t final_steps = sim.steps_done;
    for (int s = 0; s < ns; ++s) {
        MAG_CK(cudaMemcpyAsync(&final_cnt[s], sim.sp[s].cnt.p, sizeof(Counters), cudaMemcpyDeviceToHost, st));
        final_niter[s] = sim.sp[s].niter;
        final_launches[s] = sim.sp[s].launches;
    }

    // loss
    DevArray<double> d_e;
    DevArray<unsigned long long> d_n, d_n0;
    d_e.alloc(1);
    d_n.alloc(1);
    d_n0.alloc(1);
    d_e.zero(st);
    d_n.zero(st);
    d_n0.zero(st);
    std::vector<double> mass(ns);
    for (int s = 0; s < ns; ++s) {
        mass[s] = sim.sp[s].prm.mass;
        launch_adj_loss(sim.sp[s].x.p, sim.sp[s].vz.p, sim.sp[s].n_slots, 0.5 * mass[s] / kQe, d_e.p, d_n.p, st);
        launch_adj_loss(init_state[s].x.p, init_state[s].vz.p, init_state[s].n, 0.0, d_e.p, d_n0.p, st);
    }
    double e_sum = 0;
    unsigned long long n_live = 0, n0 = 0;
    MAG_CK(cudaMemcpyAsync(&e_sum, d_e.p, 8, cudaMemcpyDeviceToHost, st));
    MAG_CK(cudaMemcpyAsync(&n_live, d_n.p, 8, cudaMemcpyDeviceToHost, st));
    MAG_CK(cudaMemcpyAsync(&n0, d_n0.p, 8, cudaMemcpyDeviceToHost, st));
    MAG_CK(cudaStreamSynchronize(st));
    AdjointResult res;
    res.n0 = (int64_t)n0;
    res.n_live = (int64_t)n_live;
    res.mean_energy_eV = n_live ? e_sum / (double)n_live : 0.0;
    res.lost_fraction = n0 ? (double)(n0 - n_live) / (double)n0 : 0.0;
    res.loss = cfg.w_energy * res.mean_energy_eV + cfg.w_lost * res.lost_fraction;

    // ---- backward --------------------------------------------------------
    struct Lam {
        DevArray<float> r, z, vx, vy, vz;
    };
    std::vector<Lam> lam(ns);
    for (int s = 0; s < ns; ++s) {
        const int64_t n = sim.sp[s].n_slots;
        for (auto* a : {&lam[s].r, &lam[s].z, &lam[s].vx, &lam[s].vy, &lam[s].vz}) a->alloc(std::max<int64_t>(n, 1));
        const double coef = n_live ? cfg.w_energy * mass[s] / (kQe * (double)n_live) : 0.0;
        launch_adj_seed(sim.sp[s].x.p, sim.sp[s].vz.p, n, coef, lam[s].r.p, lam[s].z.p, lam[s].vx.p, lam[s].vy.p,
                        lam[s].vz.p, st);
    }
    std::vector<std::vector<Snap>> traj(K);
    for (auto& c : traj) c.resize(ns);
    std::vector<DevArray<double>> ustore(sc ? K : 0);

    auto adjoint_solve = [&]() {
        // g -> y = A^-T g (free nodes), lrho, voltage gradients
        launch_adj_rhs(nx, nz, sim.d_mask.p, g.p, d_wsc.p, adj_rho.p, st);
        SolveArgs a = sim.solve_args(false, 2, false);
        a.u = adj_u.p;
        a.voltage = zeros.p;
        a.rho64 = adj_rho.p;
        a.Exf = nullptr;
        a.Ezf = nullptr;
        sim.run_solve(a);
        launch_adj_post(nx, nz, sim.d_mask.p, adj_u.p, d_w.p, d_scale.p, y.p, lrho.p, st);
        launch_adj_dirichlet(nx, nz, sim.d_mask.p, g.p, y.p, sim.lv.st64.p, sim.lv.k2, d_basis.p, np, d_grad.p, st);
    };
    auto particle_adjoint = [&](int s, const Snap& before, const uint32_t* x_after, bool init, uint64_t step_niter) {
        SpeciesState& S = sim.sp[s];
        const uint64_t keep = S.niter;
        S.niter = step_niter;
        PushArgs pa = sim.push_args(s, init);
        S.niter = keep;
        pa.Exf = Exf_t.p;
        pa.Ezf = Ezf_t.p;
        AdjPushArgs d{};
        d.x0 = before.x.p;
        d.z0 = before.z.p;
        d.vx0 = before.vx.p;
        d.vy0 = before.vy.p;
        d.vz0 = before.vz.p;
        d.x1 = x_after;
        d.n = before.n;
        d.lr = lam[s].r.p;
        d.lz = lam[s].z.p;
        d.lvx = lam[s].vx.p;
        d.lvy = lam[s].vy.p;
        d.lvz = lam[s].vz.p;
        d.lExf = lExf.p;
        d.lEzf = lEzf.p;
        d.lB = cfg.grad_b ? d_grad.p + np : nullptr;
        d.init = init ? 1 : 0;
        sim.launches += launch_adj_push(pa, d, coord, st);
    };

    for (int sg = nseg - 1; sg >= 0; --sg) {
        const uint64_t n_begin = (uint64_t)sg * K;
        const int len = (int)std::min<uint64_t>((uint64_t)K, N - n_begin);
        for (int s = 0; s < ns; ++s) {
            give(ckpt[sg][s], sim.sp[s], st);
            sim.sp[s].niter = n_begin;
        }
        copy_d(sim.u64, ckpt_u[sg], nn, st);
        sim.steps_done = n_begin;
        if (sc) sim.deposit_all();
        for (int j = 0; j < len; ++j) {
            for (int s = 0; s < ns; ++s) take(traj[j][s], sim.sp[s], st);
            sim.step();
            if (sc) copy_d(ustore[j], sim.u64, nn, st);
        }
        for (int j = len - 1; j >= 0; --j) {
            const double* u_n = sc ? ustore[j].p : sim.u64.p;
            launch_faces(u_n, nx, nz, sim.dx, sim.dz, Exf_t.p, Ezf_t.p, st);
            lExf.zero(st);
            lEzf.zero(st);
            for (int s = 0; s < ns; ++s) {
                if (traj[j][s].n == 0) continue;
                const uint32_t* xa = j + 1 < len ? traj[j + 1][s].x.p : sim.sp[s].x.p;
                particle_adjoint(s, traj[j][s], xa, false, n_begin + j);
            }
            g.zero(st);
            launch_adj_faces(nx, nz, sim.dx, sim.dz, lExf.p, lEzf.p, g.p, st);
            if (sc) {
                adjoint_solve();
                for (int s = 0; s < ns; ++s)
                    if (traj[j][s].n)
                        launch_adj_deposit(traj[j][s].x.p, traj[j][s].z.p, traj[j][s].n, nx, nz, lrho.p,
                                           sim.sp[s].prm.charge, lam[s].r.p, lam[s].z.p, st);
            } else {
                launch_adj_faces(nx, nz, sim.dx, sim.dz, lExf.p, lEzf.p, g_static.p, st);
            }
        }
    }
    // the leapfrog start and the potential it used
    launch_faces(u_init.p, nx, nz, sim.dx, sim.dz, Exf_t.p, Ezf_t.p, st);
    lExf.zero(st);
    lEzf.zero(st);
    for (int s = 0; s < ns; ++s)
        if (init_state[s].n) particle_adjoint(s, init_state[s], nullptr, true, 0);
    g.zero(st);
    launch_adj_faces(nx, nz, sim.dx, sim.dz, lExf.p, lEzf.p, g.p, st);
    if (sc) {
        adjoint_solve();
    } else {
        launch_adj_faces(nx, nz, sim.dx, sim.dz, lExf.p, lEzf.p, g_static.p, st);
        if (!sim.p.electric_field_from_file) {
            copy_d(g, g_static, nn, st);
            adjoint_solve();
        }
    }
    res.grad.assign((size_t)np + nb, 0.0);
    std::vector<double> gr(np + 3);
    MAG_CK(cudaMemcpyAsync(gr.data(), d_grad.p, (np + 3) * 8, cudaMemcpyDeviceToHost, st));

    // the simulation resumes from the end of the forward run
    for (int s = 0; s < ns; ++s) {
        give(final_state[s], sim.sp[s], st);
        MAG_CK(cudaMemcpyAsync(sim.sp[s].cnt.p, &final_cnt[s], sizeof(Counters), cudaMemcpyHostToDevice, st));
        sim.sp[s].niter = final_niter[s];
        sim.sp[s].launches = final_launches[s];
    }
    copy_d(sim.u64, final_u, nn, st);
    sim.steps_done = final_steps;
    sim.sort_interval = saved_sort;
    if (sc) sim.deposit_all();
    MAG_CK(cudaStreamSynchronize(st));
    for (int q = 0; q < np + nb; ++q) res.grad[q] = gr[q];
    return res;
}

}  // namespace mag
