// Batched runs (batch.hpp): per step, one solve launch (a block per
// self-consistent instance), one persistent particle launch per kernel
// variant, one collision launch; between particle sorts the steps are replayed
// from a captured CUDA graph whose argument copies read a ring of pinned
// host buffers that the host refills before each replay.
#include "batch.hpp"

#include <algorithm>
#include <cstring>
#include <map>
#include <tuple>

#include "kernels.hpp"

namespace mag {

namespace {

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

bool has_b_field(const Sim& s) { return !s.p.magnetic_field_const || s.p.Br != 0.0 || s.p.Bt != 0.0 || s.p.Bz != 0.0; }

}  // namespace

bool Batch::Layout::operator==(const Layout& o) const
{
    return solve_off == o.solve_off && coll_off == o.coll_off && bytes == o.bytes && push_off == o.push_off &&
           chunk_off == o.chunk_off && push_items == o.push_items && key_coord == o.key_coord &&
           key_emode == o.key_emode && key_hasb == o.key_hasb && n_solve == o.n_solve && n_coll == o.n_coll &&
           max_tables == o.max_tables && solo_solve == o.solo_solve;
}

Batch::Batch(const std::vector<BatchInstanceDesc>& desc, const SimOptions& base)
{
    if (desc.empty()) throw Error(-1, "a batch needs at least one instance");
    device = base.device;
    MAG_CK(cudaSetDevice(device));
    MAG_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    if (cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sm_count < 1)
        sm_count = 1;
    cfg.push_vec = base.push_vec == 1 || base.push_vec == 2 || base.push_vec == 4 ? base.push_vec : 2;
    cfg.sort_interval = base.sort_interval == 0 ? 20 : base.sort_interval;
    sims.reserve(desc.size());
    for (size_t i = 0; i < desc.size(); ++i) {
        SimOptions o = base;
        o.seed = desc[i].seed;
        o.stream = stream;
        o.direct_solve = -1;  // the batch solves every instance with its own kernel
        try {
            sims.emplace_back(new Sim(desc[i].config, desc[i].species_conf, o));
            if (sims.back()->p.use_source)
                throw Error(-1, "batched runs: use_source (particle source boxes) is not provided; run the instance alone");
            if (sims.back()->p.u_smooth)
                throw Error(-1, "batched runs: u_smooth (potential smoothing) is not provided; run the instance alone");
            if (!desc[i].initscript.empty()) sims.back()->run_initscript(desc[i].initscript);
        } catch (const Error& e) {
            throw Error(e.code, "instance " + std::to_string(i) + ": " + e.what());
        }
    }
}

Batch::~Batch()
{
    cudaSetDevice(device);
    if (stream) cudaStreamSynchronize(stream);
    destroy_graph();
    sims.clear();
    for (auto& s : ring) {
        if (s.host) cudaFreeHost(s.host);
        if (s.dev) cudaFree(s.dev);
        if (s.done) cudaEventDestroy(s.done);
    }
    if (stream) cudaStreamDestroy(stream);
}

void Batch::destroy_graph()
{
    if (graph) cudaGraphExecDestroy(graph);
    graph = nullptr;
    graph_steps = 0;
}

void Batch::advance_init()
{
    MAG_CK(cudaSetDevice(device));
    for (auto& s : sims) s->advance_init();
}

bool Batch::sort_due() const
{
    if (cfg.sort_interval <= 0) return false;
    if (steps_done % (uint64_t)cfg.sort_interval == 0) return true;
    for (auto& s : sims)
        if (s->sort_due) return true;
    return false;
}

void Batch::sort_all()
{
    for (auto& s : sims) {
        for (size_t k = 0; k < s->sp.size(); ++k) s->sort_species((int)k);
        s->sort_due = false;
    }
}

Batch::Layout Batch::plan() const
{
    Layout L;
    size_t off = 0;
    // solves
    for (int i = 0; i < (int)sims.size(); ++i) {
        const Sim& s = *sims[i];
        if (!s.p.selfconsistent) continue;
        if ((long long)s.nx * s.nz <= kSingleBlockNodes) ++L.n_solve;
        else L.solo_solve.push_back(i);
    }
    L.solve_off = off;
    off = align256(off + (size_t)L.n_solve * sizeof(SolveArgs));
    // particle work items grouped by kernel variant
    std::map<std::tuple<int, int, int>, int> keys;
    for (auto& sp : sims) {
        const Sim& s = *sp;
        const int coord = s.p.coord == CYLINDRICAL ? 1 : 0, hb = has_b_field(s) ? 1 : 0;
        for (size_t k = 0; k < s.sp.size(); ++k) {
            if (s.sp[k].n_slots == 0) continue;
            auto key = std::make_tuple(coord, s.emode, hb);
            auto it = keys.find(key);
            if (it == keys.end()) {
                keys[key] = (int)L.push_items.size();
                L.push_items.push_back(0);
                L.key_coord.push_back(coord);
                L.key_emode.push_back(s.emode);
                L.key_hasb.push_back(hb);
            }
            ++L.push_items[keys[key]];
            if (s.sp[k].threshold != 0) {
                ++L.n_coll;
                L.max_tables = std::max(L.max_tables, (int)s.d_tables.n);
            }
        }
    }
    for (size_t q = 0; q < L.push_items.size(); ++q) {
        L.push_off.push_back(off);
        off = align256(off + (size_t)L.push_items[q] * sizeof(PushArgs));
        L.chunk_off.push_back(off);
        off = align256(off + (size_t)(L.push_items[q] + 1) * sizeof(unsigned));
    }
    L.coll_off = off;
    off = align256(off + (size_t)L.n_coll * sizeof(CollideArgs));
    L.bytes = off;
    return L;
}

void Batch::pack(const Layout& L, Slot& slot)
{
    unsigned char* h = slot.host;
    SolveArgs* sa = reinterpret_cast<SolveArgs*>(h + L.solve_off);
    CollideArgs* ca = reinterpret_cast<CollideArgs*>(h + L.coll_off);
    std::vector<int> fill(L.push_items.size(), 0);
    int nc = 0;
    const int chunk = push_batch_chunk(cfg.push_vec);
    // solve blocks largest grid first, so that the small instances fill the
    // second wave of blocks instead of starting large ones late
    std::vector<std::pair<long long, SolveArgs>> solves;
    for (auto& sp : sims) {
        Sim& s = *sp;
        if (s.p.selfconsistent && (long long)s.nx * s.nz <= kSingleBlockNodes) {
            solves.emplace_back((long long)s.nx * s.nz, s.solve_args(false, s.rho_override ? 2 : 1, true));
            solves.back().second.prof = nullptr;  // one block per instance: no phase timing
            s.rho_override = false;
        }
    }
    std::stable_sort(solves.begin(), solves.end(),
                     [](const auto& x, const auto& y) { return x.first > y.first; });
    for (size_t q = 0; q < solves.size(); ++q) sa[q] = solves[q].second;
    for (auto& sp : sims) {
        Sim& s = *sp;
        const int coord = s.p.coord == CYLINDRICAL ? 1 : 0, hb = has_b_field(s) ? 1 : 0;
        int q = 0;
        for (; q < (int)L.push_items.size(); ++q)
            if (L.key_coord[q] == coord && L.key_emode[q] == s.emode && L.key_hasb[q] == hb) break;
        for (size_t k = 0; k < s.sp.size(); ++k) {
            SpeciesState& S = s.sp[k];
            if (S.n_slots == 0) continue;
            PushArgs pa = s.push_args((int)k, false);
            pa.slot = (int)(S.launches & 1);
            pa.fold_slot = S.launches > 0 ? (int)((S.launches - 1) & 1) : -1;
            PushArgs* pq = reinterpret_cast<PushArgs*>(h + L.push_off[q]);
            unsigned* off = reinterpret_cast<unsigned*>(h + L.chunk_off[q]);
            const int f = fill[q]++;
            pq[f] = pa;
            if (f == 0) off[0] = 0;
            off[f + 1] = off[f] + (unsigned)((S.n_slots + chunk - 1) / chunk);
            if (S.threshold != 0) {
                CollideArgs c = s.collide_args((int)k);
                c.slot = pa.slot;
                ca[nc++] = c;
            }
        }
    }
    // the step is issued: host counters advance as in Sim::step
    for (auto& sp : sims) {
        Sim& s = *sp;
        for (auto& S : s.sp) {
            if (S.n_slots > 0) S.launches++;
            S.niter++;
        }
        s.steps_done++;
    }
    steps_done++;
}

void Batch::launch_step(const Layout& L, const Slot& slot)
{
    MAG_CK(cudaMemcpyAsync(slot.dev, slot.host, L.bytes, cudaMemcpyHostToDevice, stream));
    for (int i : L.solo_solve) sims[i]->solve(false, sims[i]->rho_override ? 2 : 1, true, false);
    launches += launch_solve_batch(reinterpret_cast<const SolveArgs*>(slot.dev + L.solve_off), L.n_solve,
                                   cfg.solve_threads, stream);
    for (size_t q = 0; q < L.push_items.size(); ++q)
        launches += launch_push_batch(reinterpret_cast<const PushArgs*>(slot.dev + L.push_off[q]),
                                      reinterpret_cast<const unsigned*>(slot.dev + L.chunk_off[q]), L.push_items[q],
                                      L.key_coord[q], L.key_emode[q], L.key_hasb[q] != 0, cfg.push_vec, sm_count,
                                      stream);
    launches += launch_collide_batch(reinterpret_cast<const CollideArgs*>(slot.dev + L.coll_off), L.n_coll,
                                     L.max_tables, stream);
}

void Batch::ensure_ring(size_t count, size_t bytes)
{
    for (auto& s : ring)
        if (s.cap < bytes) {
            MAG_CK(cudaStreamSynchronize(stream));
            destroy_graph();  // captured copies point at the old buffers
            if (s.host) cudaFreeHost(s.host);
            if (s.dev) cudaFree(s.dev);
            s.host = nullptr;
            s.dev = nullptr;
            MAG_CK(cudaMallocHost((void**)&s.host, bytes));
            MAG_CK(cudaMalloc((void**)&s.dev, bytes));
            s.cap = bytes;
        }
    while (ring.size() < count) {
        Slot s;
        MAG_CK(cudaMallocHost((void**)&s.host, bytes));
        MAG_CK(cudaMalloc((void**)&s.dev, bytes));
        MAG_CK(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
        s.cap = bytes;
        ring.push_back(s);
    }
}

Batch::Slot& Batch::take_slot(size_t bytes)
{
    ensure_ring(4, bytes);
    if (graph_inflight) {
        MAG_CK(cudaStreamSynchronize(stream));
        graph_inflight = false;
    }
    Slot& s = ring[ring_next++ % 4];
    MAG_CK(cudaEventSynchronize(s.done));  // the copy out of this buffer has run
    return s;
}

void Batch::advance(uint64_t nsteps)
{
    MAG_CK(cudaSetDevice(device));
    while (nsteps > 0) {
        if (sort_due()) sort_all();
        uint64_t g = nsteps;
        if (cfg.sort_interval > 0) {
            const uint64_t to_sort = (uint64_t)cfg.sort_interval - steps_done % (uint64_t)cfg.sort_interval;
            g = std::min(g, to_sort);
        }
        const Layout L = plan();
        const bool fresh = !graph || graph_steps != (int)g - 1 || !(L == graph_layout);
        // a graph is (re)captured after one ordinary step of the same layout has
        // run, so every kernel it contains is loaded and configured beforehand
        const uint64_t plain = !use_graph || g < 3 || !L.solo_solve.empty() ? g : (fresh ? 1 : 0);
        if (plain > 0 && graph_inflight) {
            MAG_CK(cudaStreamSynchronize(stream));  // the replay no longer reads the ring
            graph_inflight = false;
        }
        for (uint64_t k = 0; k < plain; ++k) {
            Slot& s = take_slot(L.bytes);
            pack(L, s);
            launch_step(L, s);
            MAG_CK(cudaEventRecord(s.done, stream));
        }
        if (plain < g) {
            const size_t G = (size_t)(g - plain);
            MAG_CK(cudaStreamSynchronize(stream));  // no copy out of the ring is pending
            graph_inflight = false;
            ensure_ring(std::max<size_t>(G, 4), L.bytes);
            for (size_t k = 0; k < G; ++k) pack(L, ring[k]);
            if (!graph || graph_steps != (int)G || !(L == graph_layout)) {
                destroy_graph();
                cudaGraph_t gr = nullptr;
                MAG_CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
                for (size_t k = 0; k < G; ++k) launch_step(L, ring[k]);
                MAG_CK(cudaStreamEndCapture(stream, &gr));
                const cudaError_t e = cudaGraphInstantiate(&graph, gr, 0);
                cudaGraphDestroy(gr);
                MAG_CK(e);
                graph_layout = L;
                graph_steps = (int)G;
            }
            MAG_CK(cudaGraphLaunch(graph, stream));
            graph_inflight = true;
        }
        nsteps -= g;
    }
    MAG_CK(cudaGetLastError());
}

BatchTuning Batch::tune(int steps_per_trial)
{
    MAG_CK(cudaSetDevice(device));
    if (steps_per_trial < 1) steps_per_trial = 3;
    const bool graph_was = use_graph;
    use_graph = false;
    cudaEvent_t e0, e1;
    MAG_CK(cudaEventCreate(&e0));
    MAG_CK(cudaEventCreate(&e1));
    auto trial = [&](int steps) {
        advance(1);  // settle (sorts, first-use set-up) outside the timed steps
        MAG_CK(cudaEventRecord(e0, stream));
        advance((uint64_t)steps);
        MAG_CK(cudaEventRecord(e1, stream));
        MAG_CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        MAG_CK(cudaEventElapsedTime(&ms, e0, e1));
        return (double)ms / steps;
    };
    BatchTuning best = cfg;
    best.ms_per_step = 1e30;
    for (int th : {256, 512, 1024}) {
        cfg.solve_threads = th;
        const double t = trial(steps_per_trial);
        if (t < best.ms_per_step) {
            best.ms_per_step = t;
            best.solve_threads = th;
        }
    }
    cfg.solve_threads = best.solve_threads;
    for (int v : {1, 2, 4}) {
        cfg.push_vec = v;
        const double t = trial(steps_per_trial);
        if (t < best.ms_per_step) {
            best.ms_per_step = t;
            best.push_vec = v;
        }
    }
    cfg.push_vec = best.push_vec;
    // the sort interval: time a whole interval of each candidate (sort included)
    double best_sort = 1e30;
    for (int si : {10, 20, 50}) {
        cfg.sort_interval = si;
        const double t = trial(si);
        if (t < best_sort) {
            best_sort = t;
            best.sort_interval = si;
        }
    }
    cfg = best;
    cfg.ms_per_step = best_sort;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    use_graph = graph_was;
    destroy_graph();
    return cfg;
}

int Batch::sync()
{
    MAG_CK(cudaSetDevice(device));
    MAG_CK(cudaStreamSynchronize(stream));
    int err = 0;
    for (auto& s : sims) {
        const int e = s->sync();
        if (e && !err) err = e;
    }
    return err;
}

}  // namespace mag
