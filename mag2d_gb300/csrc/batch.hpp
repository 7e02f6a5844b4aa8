// Batched runs: many independent simulation instances (uneven grids,
// particle counts and pressures) advanced together, each step as a handful of
// launches that cover every instance — one block per instance for the
// Poisson solves, one persistent grid over all instances' particles, one
// block per colliding species for the scatter — optionally replayed from a
// captured CUDA graph between particle sorts.  Launch parameters (slots per
// thread, solve block size, sort interval) are picked by timing real steps
// (Batch::tune); none of them changes results.
#pragma once

#include <cuda_runtime.h>

#include <memory>
#include <string>
#include <vector>

#include "sim.hpp"

namespace mag {

struct BatchInstanceDesc {
    std::string config, species_conf, initscript;
    uint64_t seed = 1;
};

struct BatchTuning {
    int push_vec = 2;        // slots per thread of the particle kernel
    int solve_threads = 512; // threads of each instance's solve block
    int sort_interval = 20;  // steps between particle sorts
    double ms_per_step = 0;  // measured with the chosen parameters
};

class Batch {
public:
    Batch(const std::vector<BatchInstanceDesc>& desc, const SimOptions& base);
    ~Batch();
    Batch(const Batch&) = delete;
    Batch& operator=(const Batch&) = delete;

    void advance_init();
    void advance(uint64_t nsteps);
    // time candidate launch parameters on real steps (steps_per_trial each), keep the fastest
    BatchTuning tune(int steps_per_trial);
    int sync();  // first device error code of any instance (0 = none)

    int size() const { return (int)sims.size(); }
    Sim& instance(int i) { return *sims[i]; }

    cudaStream_t stream = nullptr;
    int device = 0;
    BatchTuning cfg;
    bool use_graph = true;
    uint64_t steps_done = 0;
    int64_t launches = 0;

private:
    std::vector<std::unique_ptr<Sim>> sims;
    int sm_count = 1;

    // one step's arguments, packed for a single host-to-device copy
    struct Layout {
        size_t solve_off = 0, coll_off = 0, bytes = 0;
        std::vector<size_t> push_off, chunk_off;     // per kernel key
        std::vector<int> push_items;                 // per kernel key
        std::vector<int> key_coord, key_emode, key_hasb;
        int n_solve = 0, n_coll = 0, max_tables = 0;
        std::vector<int> solo_solve;                 // instances whose grid needs a multi-block solve
        bool operator==(const Layout& o) const;
    };
    struct Slot {
        unsigned char* host = nullptr;  // pinned
        unsigned char* dev = nullptr;
        size_t cap = 0;
        cudaEvent_t done = nullptr;     // last copy out of this slot finished
    };
    std::vector<Slot> ring;
    size_t ring_next = 0;
    cudaGraphExec_t graph = nullptr;
    Layout graph_layout;
    int graph_steps = 0;
    bool graph_inflight = false;  // a replay may still read the ring
    std::vector<size_t> graph_slots;

    bool sort_due() const;
    void sort_all();
    Layout plan() const;
    // fill slot with the arguments of the next step (advancing the host step counters)
    void pack(const Layout& L, Slot& slot);
    void launch_step(const Layout& L, const Slot& slot);
    Slot& take_slot(size_t bytes);
    void ensure_ring(size_t count, size_t bytes);
    void destroy_graph();
};

}  // namespace mag
