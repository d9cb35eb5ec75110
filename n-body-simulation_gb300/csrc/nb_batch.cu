// nb_batch.cu -- ensembles of independent systems of uneven size in one persistent launch
// (the one-sided kernel of nb_pair.cuh or the symmetric kernel of nb_pair_sym.cu), the tile
// autotuner over both kernels' shapes, and CUDA-graph capture of whole leapfrog steps.
//
// All systems live in concatenated FP64 arrays; system s owns bodies [off_s, off_s + count_s).
// Forces never cross systems. The batch pre-allocates every buffer its launches use (plan,
// FP32 sources/targets, partials for the largest configuration), so a step can be captured
// into a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "nb_pair.cuh"
#include "nb_pair_sym.cuh"

namespace {
// Batch configurations: 0 .. NB_PAIR_CONFIGS-1 the one-sided pair kernel's tile shapes, then
// NB_SYM_CONFIGS shapes of the symmetric kernel (each unordered pair once, both bodies).
constexpr int NB_BATCH_CONFIGS = nb::NB_PAIR_CONFIGS + nb::NB_SYM_CONFIGS;
inline bool is_sym(int cfg) { return cfg >= nb::NB_PAIR_CONFIGS; }
}  // namespace

struct nb_batch {
    int device = 0;
    uint32_t n_systems = 0;
    uint32_t n_total = 0;
    int cfg = 0;
    std::vector<uint32_t> counts;
    void* mem = nullptr;
    uint32_t *sys_off = nullptr, *tgt_begin = nullptr, *t_off = nullptr, *ib_off = nullptr;
    uint64_t* unit_off = nullptr;
    nbpair::SrcDup* src = nullptr;
    float4* tgt = nullptr;
    float* part = nullptr;
    size_t part_floats = 0;
    nbpair::Plan plan{};
    // symmetric kernel: per-system table, padded FP32 records, i-side and j-side partials
    nbsym::SymSys* sym_table = nullptr;
    float4* sym_src = nullptr;
    float* sym_part_i = nullptr;
    float* sym_part_j = nullptr;
    nbsym::SymPlan sym_plan{};
};


namespace {

struct HostPlan {
    std::vector<uint64_t> unit_off;
    std::vector<uint32_t> ib_off;
    uint32_t ctas = 0;
    uint64_t units = 0;
};

nb_status host_plan(const nb_batch* b, int cfg, int sm_count, HostPlan* hp) {
    const nb::PairConfig& C = nb::kPairConfigs[cfg];
    const uint32_t ib = (uint32_t)(C.threads * C.ip);
    hp->unit_off.assign(b->n_systems + 1, 0);
    hp->ib_off.assign(b->n_systems + 1, 0);
    for (uint32_t s = 0; s < b->n_systems; ++s) {
        const uint32_t n = b->counts[s];
        const uint32_t n_ib = (n + ib - 1) / ib, n_jt = (n + C.jt - 1) / C.jt;
        hp->unit_off[s + 1] = hp->unit_off[s] + (uint64_t)n_ib * n_jt;
        hp->ib_off[s + 1] = hp->ib_off[s] + n_ib;
    }
    int per_sm = 0;
    NB_TRY(nb::pair_ctas_per_sm(cfg, &per_sm));
    hp->units = hp->unit_off[b->n_systems];
    uint64_t ctas = (uint64_t)sm_count * per_sm;
    if (ctas > hp->units) ctas = hp->units;
    hp->ctas = (uint32_t)(ctas ? ctas : 1);
    return NB_OK;
}

nb_status apply_config(nb_batch* b, int cfg, int sm_count) {
    if (is_sym(cfg)) {
        nb::SymHostPlan sp;
        NB_TRY(nb::sym_host_plan(nb::SYM_F32, cfg - nb::NB_PAIR_CONFIGS, b->counts.data(),
                                 b->n_systems, sm_count, &sp));
        NB_CUDA_TRY(cudaMemcpy(b->sym_table, sp.sys.data(), sp.sys.size() * sizeof(nbsym::SymSys),
                               cudaMemcpyHostToDevice));
        b->sym_plan.sys = b->sym_table;
        b->sym_plan.n_systems = b->n_systems;
        b->sym_plan.ctas = sp.ctas;
        b->sym_plan.n_total = sp.n_total;
        b->sym_plan.n_records = sp.n_records;
        b->sym_plan.units = sp.units;
        b->cfg = cfg;
        return NB_OK;
    }
    HostPlan hp;
    NB_TRY(host_plan(b, cfg, sm_count, &hp));
    NB_CUDA_TRY(cudaMemcpy(b->unit_off, hp.unit_off.data(), hp.unit_off.size() * 8,
                           cudaMemcpyHostToDevice));
    NB_CUDA_TRY(cudaMemcpy(b->ib_off, hp.ib_off.data(), hp.ib_off.size() * 4, cudaMemcpyHostToDevice));
    b->cfg = cfg;
    b->plan.ctas = hp.ctas;
    b->plan.units = hp.units;
    return NB_OK;
}

nb_status batch_accel(nb_ctx* ctx, nb_batch* b, const double* m, const double* x, const double* y,
                      const double* z, double* ax, double* ay, double* az, double G, double eps2,
                      cudaStream_t s) {
    if (is_sym(b->cfg)) {
        nbsym::SymPlan S = b->sym_plan;
        S.wait_limit = ctx->wait_limit;
        return nb::sym_launch(nb::SYM_F32, b->cfg - nb::NB_PAIR_CONFIGS, S, m, x, y, z, G, eps2,
                              b->sym_src, b->sym_part_i, b->sym_part_j, ax, ay, az,
                              ctx->dev_error, s);
    }
    if (b->plan.units == 0) return NB_OK;
    nbpair::Plan P = b->plan;
    P.wait_limit = ctx->wait_limit;
    return nb::pair_launch(b->cfg, P, m, x, y, z, b->n_total, b->n_total, G, eps2, b->src,
                           b->tgt, b->part, ax, ay, az, ctx->dev_error, s);
}

}  // namespace

extern "C" {

nb_status nb_batch_create(nb_ctx* ctx, uint32_t n_systems, const uint32_t* counts,
                          nb_batch** out) {
    NB_CHECK_CTX(ctx);
    if (!out || !counts || n_systems == 0)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_batch_create: bad arguments");
    *out = nullptr;
    nb_batch* b = new nb_batch();
    b->device = ctx->device;
    b->n_systems = n_systems;
    b->counts.assign(counts, counts + n_systems);
    std::vector<uint32_t> off(n_systems + 1, 0);
    for (uint32_t s = 0; s < n_systems; ++s) {
        const uint64_t next = (uint64_t)off[s] + counts[s];
        if (next > 0xffffffffull) {
            delete b;
            return nb::set_error(NB_ERR_INVALID_ARG, "nb_batch_create: more than 2^32 bodies");
        }
        off[s + 1] = (uint32_t)next;
    }
    b->n_total = off[n_systems];
    // partial buffer large enough for every configuration
    size_t part_floats = 0;
    for (int c = 0; c < nb::NB_PAIR_CONFIGS; ++c) {
        HostPlan hp;
        nb_status st = host_plan(b, c, ctx->sm_count, &hp);
        if (st != NB_OK) {
            delete b;
            return st;
        }
        const size_t f = nb::pair_partial_floats(c, hp.ctas, hp.ib_off[n_systems]);
        if (f > part_floats) part_floats = f;
    }
    b->part_floats = part_floats;
    // symmetric configurations: the largest records and partials of any of them
    size_t sym_records = 0, sym_pi = 0, sym_pj = 0;
    for (int c = 0; c < nb::NB_SYM_CONFIGS; ++c) {
        nb::SymHostPlan sp;
        nb_status st =
            nb::sym_host_plan(nb::SYM_F32, c, b->counts.data(), n_systems, ctx->sm_count, &sp);
        if (st != NB_OK) {
            delete b;
            return st;
        }
        sym_records = std::max(sym_records, (size_t)sp.n_records);
        sym_pi = std::max(sym_pi, nb::sym_part_i_bytes(nb::SYM_F32, c, sp.ctas, sp.n_blocks));
        sym_pj = std::max(sym_pj, nb::sym_part_j_bytes(nb::SYM_F32, c, sp.units));
    }
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t ns = n_systems + 1;
    const size_t sizes[] = {al(ns * 4), al(ns * 4), al(ns * 4), al(ns * 4), al(ns * 8),
                            al((size_t)b->n_total * sizeof(nbpair::SrcDup) + 32),
                            al((size_t)b->n_total * sizeof(float4) + 16), al(part_floats * 4),
                            al(ns * sizeof(nbsym::SymSys)), al(sym_records * sizeof(float4)),
                            al(sym_pi), al(sym_pj)};
    size_t total = 0;
    for (size_t v : sizes) total += v;
    cudaError_t e = cudaMalloc(&b->mem, total);
    if (e != cudaSuccess) {
        delete b;
        return nb::cuda_error(e, "nb_batch_create");
    }
    char* p = (char*)b->mem;
    b->sys_off = (uint32_t*)p; p += sizes[0];
    b->tgt_begin = (uint32_t*)p; p += sizes[1];
    b->t_off = (uint32_t*)p; p += sizes[2];
    b->ib_off = (uint32_t*)p; p += sizes[3];
    b->unit_off = (uint64_t*)p; p += sizes[4];
    b->src = (nbpair::SrcDup*)p; p += sizes[5];
    b->tgt = (float4*)p; p += sizes[6];
    b->part = (float*)p; p += sizes[7];
    b->sym_table = (nbsym::SymSys*)p; p += sizes[8];
    b->sym_src = (float4*)p; p += sizes[9];
    b->sym_part_i = (float*)p; p += sizes[10];
    b->sym_part_j = (float*)p;
    std::vector<uint32_t> zeros(n_systems, 0);
    e = cudaMemcpy(b->sys_off, off.data(), ns * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->t_off, off.data(), ns * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->tgt_begin, zeros.data(), n_systems * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(b->mem);
        delete b;
        return nb::cuda_error(e, "nb_batch_create");
    }
    b->plan.n_systems = n_systems;
    b->plan.sys_off = b->sys_off;
    b->plan.tgt_begin = b->tgt_begin;
    b->plan.t_off = b->t_off;
    b->plan.unit_off = b->unit_off;
    b->plan.ib_off = b->ib_off;
    nb_status st = apply_config(b, 0, ctx->sm_count);
    if (st != NB_OK) {
        cudaFree(b->mem);
        delete b;
        return st;
    }
    *out = b;
    return NB_OK;
}

nb_status nb_batch_destroy(nb_batch* b) {
    if (!b) return NB_OK;
    if (b->mem) cudaFree(b->mem);
    delete b;
    return NB_OK;
}

nb_status nb_batch_info(const nb_batch* b, uint32_t* n_total, int* config, int* threads,
                        int* targets_per_thread, int* j_tile) {
    if (!b) return nb::set_error(NB_ERR_INVALID_ARG, "nb_batch_info: null batch");
    int t = 0, ip = 0, jt = 0;
    if (is_sym(b->cfg)) {
        const nb::SymConfig& C = nb::kSymConfigs[b->cfg - nb::NB_PAIR_CONFIGS];
        t = 32 * C.warps;
        ip = C.p;
        jt = C.jt;
    } else {
        const nb::PairConfig& C = nb::kPairConfigs[b->cfg];
        t = C.threads;
        ip = C.ip;
        jt = C.jt;
    }
    if (n_total) *n_total = b->n_total;
    if (config) *config = b->cfg;
    if (threads) *threads = t;
    if (targets_per_thread) *targets_per_thread = ip;
    if (j_tile) *j_tile = jt;
    return NB_OK;
}

nb_status nb_batch_set_config(nb_ctx* ctx, nb_batch* b, int config) {
    NB_CHECK_CTX(ctx);
    if (!b || config < 0 || config >= NB_BATCH_CONFIGS)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_batch_set_config: bad arguments");
    return apply_config(b, config, ctx->sm_count);
}

nb_status nb_batch_naive_accel(nb_ctx* ctx, nb_batch* b, const double* m, const double* x,
                               const double* y, const double* z, double* ax, double* ay,
                               double* az, double G, double eps2, nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (!b || !m || !x || !y || !z || !ax || !ay || !az)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_batch_naive_accel: null argument");
    return batch_accel(ctx, b, m, x, y, z, ax, ay, az, G, eps2, (cudaStream_t)stream);
}

nb_status nb_batch_autotune(nb_ctx* ctx, nb_batch* b, const double* m, const double* x,
                            const double* y, const double* z, double* ax, double* ay, double* az,
                            double G, double eps2, int reps, float* ms_per_config, int* chosen) {
    NB_CHECK_CTX(ctx);
    if (!b || reps < 1) return nb::set_error(NB_ERR_INVALID_ARG, "nb_batch_autotune: bad arguments");
    cudaEvent_t e0, e1;
    NB_CUDA_TRY(cudaEventCreate(&e0));
    NB_CUDA_TRY(cudaEventCreate(&e1));
    int best = 0;
    float best_ms = 0;
    nb_status st = NB_OK;
    for (int c = 0; c < NB_BATCH_CONFIGS && st == NB_OK; ++c) {
        st = apply_config(b, c, ctx->sm_count);
        if (st != NB_OK) break;
        st = batch_accel(ctx, b, m, x, y, z, ax, ay, az, G, eps2, nullptr);  // warm-up
        if (st != NB_OK) break;
        cudaEventRecord(e0);
        for (int r = 0; r < reps && st == NB_OK; ++r)
            st = batch_accel(ctx, b, m, x, y, z, ax, ay, az, G, eps2, nullptr);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess) st = nb::check_launch("autotune");
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= reps;
        if (ms_per_config) ms_per_config[c] = ms;
        if (c == 0 || ms < best_ms) {
            best = c;
            best_ms = ms;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != NB_OK) return st;
    NB_TRY(apply_config(b, best, ctx->sm_count));
    if (chosen) *chosen = best;
    return nb_sync(ctx, nullptr);
}

// Captures `steps` leapfrog steps (kick-drift, batch accelerations, kick) into a CUDA graph.
nb_status nb_batch_graph_create(nb_ctx* ctx, nb_batch* b, const double* m, double* x, double* y,
                                double* z, double* vx, double* vy, double* vz, double* vhx,
                                double* vhy, double* vhz, double* ax, double* ay, double* az,
                                double G, double eps2, double dt, int steps, nb_graph** out) {
    NB_CHECK_CTX(ctx);
    if (!b || !out || steps < 1)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_batch_graph_create: bad arguments");
    *out = nullptr;
    cudaStream_t s;
    NB_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    nb_status st = NB_OK;
    cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s);
        return nb::cuda_error(e, "cudaStreamBeginCapture");
    }
    for (int k = 0; k < steps && st == NB_OK; ++k) {
        st = nb_leapfrog_kick_drift(ctx, vhx, vhy, vhz, vx, vy, vz, x, y, z, ax, ay, az, b->n_total,
                                    dt, (nb_stream_t)s);
        if (st == NB_OK) st = batch_accel(ctx, b, m, x, y, z, ax, ay, az, G, eps2, s);
        if (st == NB_OK)
            st = nb_leapfrog_kick(ctx, vx, vy, vz, vhx, vhy, vhz, ax, ay, az, b->n_total, dt,
                                  (nb_stream_t)s);
    }
    return nb_finish_capture(s, st, steps, out);
}

}  // extern "C"

nb_status nb_finish_capture(cudaStream_t s, nb_status st, int steps, nb_graph** out) {
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    cudaStreamDestroy(s);
    if (st != NB_OK) {
        if (graph) cudaGraphDestroy(graph);
        return st;
    }
    if (e != cudaSuccess) return nb::cuda_error(e, "cudaStreamEndCapture");
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        return nb::cuda_error(e, "cudaGraphInstantiate");
    }
    nb_graph* g = new nb_graph();
    g->graph = graph;
    g->exec = exec;
    g->steps = steps;
    *out = g;
    return NB_OK;
}

extern "C" {

nb_status nb_graph_launch(nb_graph* g, nb_stream_t stream) {
    if (!g) return nb::set_error(NB_ERR_INVALID_ARG, "nb_graph_launch: null graph");
    NB_CUDA_TRY(cudaGraphLaunch(g->exec, (cudaStream_t)stream));
    return NB_OK;
}

nb_status nb_graph_destroy(nb_graph* g) {
    if (!g) return NB_OK;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return NB_OK;
}

}  // extern "C"
