// nb_bh_export.cu -- synchronous host-side views of a built tree: statistics and the reference's
// linearised layout (BarnesHutOctree.hpp:33-95) for parity checks.
#include <cmath>
#include <deque>
#include <vector>

#include "nb_bh.cuh"

namespace {

struct HostTree {
    uint32_t n = 0, nodes = 0;
    double box[10];
    std::vector<uint8_t> level;
    std::vector<uint32_t> first, skip, body, count, ids;
    std::vector<double> comx, comy, comz, mass;
    std::vector<uint64_t> key0, key1;
};

template <typename T>
nb_status fetch(std::vector<T>& v, const T* src, size_t count) {
    v.resize(count);
    if (count) NB_CUDA_TRY(cudaMemcpy(v.data(), src, count * sizeof(T), cudaMemcpyDeviceToHost));
    return NB_OK;
}

nb_status fetch_tree(nb_bh_tree* t, HostTree& h, bool full) {
    if (!t) return nb::set_error(NB_ERR_INVALID_ARG, "null tree");
    if (!t->built) return nb::set_error(NB_ERR_NOT_BUILT, "tree not built");
    NB_CUDA_TRY(cudaSetDevice(t->device));
    NB_CUDA_TRY(cudaDeviceSynchronize());
    h.n = t->n;
    NB_CUDA_TRY(cudaMemcpy(&h.nodes, t->info, sizeof(uint32_t), cudaMemcpyDeviceToHost));
    NB_CUDA_TRY(cudaMemcpy(h.box, t->box, sizeof(h.box), cudaMemcpyDeviceToHost));
    NB_TRY(fetch(h.level, t->node_level, h.nodes));
    NB_TRY(fetch(h.body, t->node_body, h.nodes));
    NB_TRY(fetch(h.skip, t->node_skip, h.nodes));
    NB_TRY(fetch(h.ids, t->ids, h.n));
    if (full) {
        NB_TRY(fetch(h.first, t->node_first, h.nodes));
        NB_TRY(fetch(h.count, t->node_count, h.nodes));
        NB_TRY(fetch(h.comx, t->node_comx, h.nodes));
        NB_TRY(fetch(h.comy, t->node_comy, h.nodes));
        NB_TRY(fetch(h.comz, t->node_comz, h.nodes));
        NB_TRY(fetch(h.mass, t->node_mass, h.nodes));
        NB_TRY(fetch(h.key0, t->key0, h.n));
        NB_TRY(fetch(h.key1, t->key1, h.n));
    }
    return NB_OK;
}

// Parent level of every node (-1 for the top node), from the DFS order and skip links.
std::vector<int> parent_levels(const HostTree& h) {
    std::vector<int> pl(h.nodes, -1);
    std::vector<uint32_t> stack;  // open ancestors
    for (uint32_t k = 0; k < h.nodes; ++k) {
        while (!stack.empty() && h.skip[stack.back()] <= k) stack.pop_back();
        pl[k] = stack.empty() ? -1 : (int)h.level[stack.back()];
        if (h.body[k] == NB_NONE) stack.push_back(k);
    }
    return pl;
}

uint32_t digit_at(const HostTree& h, uint32_t pos, int L) {
    if (L < NB_KEY_LEVELS) return (uint32_t)(h.key0[pos] >> (60 - 3 * L)) & 7u;
    return (uint32_t)(h.key1[pos] >> (60 - 3 * (L - NB_KEY_LEVELS))) & 7u;
}

}  // namespace

extern "C" {

nb_status nb_bh_tree_stats(nb_bh_tree* t, nb_bh_stats* out) {
    if (!out) return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_tree_stats: null output");
    HostTree h;
    NB_TRY(fetch_tree(t, h, false));
    out->n = h.n;
    out->node_count = h.nodes;
    uint32_t maxd = 0;
    for (uint32_t k = 0; k < h.nodes; ++k) maxd = h.level[k] > maxd ? h.level[k] : maxd;
    out->max_depth = maxd;
    const std::vector<int> pl = parent_levels(h);
    uint64_t cells = 0;  // internal cells of the reference's tree (chains included)
    for (uint32_t k = 0; k < h.nodes; ++k)
        if (h.body[k] == NB_NONE) cells += (uint64_t)(h.level[k] - pl[k]);
    const uint64_t ref = 1 + 8 * cells;
    out->ref_node_count = ref > 0xffffffffull ? 0xffffffffu : (uint32_t)ref;
    for (int i = 0; i < 7; ++i) out->aabb[i] = h.box[i];
    return NB_OK;
}

nb_status nb_bh_export_order(nb_bh_tree* t, uint32_t* ids_in_dfs_order, uint32_t* leaf_level) {
    HostTree h;
    NB_TRY(fetch_tree(t, h, false));
    if (ids_in_dfs_order)
        for (uint32_t p = 0; p < h.n; ++p) ids_in_dfs_order[p] = h.ids[p];
    if (leaf_level)
        for (uint32_t k = 0; k < h.nodes; ++k)
            if (h.body[k] != NB_NONE) leaf_level[h.body[k]] = h.level[k];
    return NB_OK;
}

nb_status nb_bh_export_ref_layout(nb_bh_tree* t, nb_bh_ref_layout* out) {
    if (!out) return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_export_ref_layout: null output");
    HostTree h;
    NB_TRY(fetch_tree(t, h, true));
    const std::vector<int> pl = parent_levels(h);
    uint64_t cells = 0;
    for (uint32_t k = 0; k < h.nodes; ++k)
        if (h.body[k] == NB_NONE) cells += (uint64_t)(h.level[k] - pl[k]);
    const uint64_t total = 1 + 8 * cells;
    out->node_count = (uint32_t)total;
    if (total > out->capacity)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_export_ref_layout: capacity %u < %llu nodes",
                             out->capacity, (unsigned long long)total);
    if (!out->octants || !out->edge || !out->min_x || !out->min_y || !out->min_z ||
        !out->body_of_node || !out->node_is_leaf || !out->sum_masses || !out->com_x ||
        !out->com_y || !out->com_z || !out->body_count || !out->sorted_bodies)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_bh_export_ref_layout: null array");
    const uint32_t cap = out->capacity;
    // children of each compressed internal node, by octant
    std::vector<uint32_t> child(8 * (size_t)h.nodes, NB_NONE);
    for (uint32_t k = 0; k < h.nodes; ++k) {
        if (h.body[k] != NB_NONE) continue;
        for (uint32_t c = k + 1; c < h.skip[k]; c = h.skip[c])
            child[8 * (size_t)k + nb_octant_of_visit(digit_at(h, h.first[c], h.level[k]))] = c;
    }
    struct Cell {
        uint32_t id;   // reference node id
        uint32_t X;    // compressed node holding the cell's bodies (NB_NONE: empty)
        int level;
        double mnx, mny, mnz;
    };
    static const uint32_t slot_octant[8] = {5, 7, 4, 6, 1, 3, 0, 2};
    const double E = h.box[6];
    std::deque<Cell> q;
    q.push_back(Cell{0, h.nodes ? 0u : NB_NONE, 0, h.box[0], h.box[1], h.box[2]});
    uint32_t next_free = 1;
    while (!q.empty()) {
        const Cell c = q.front();
        q.pop_front();
        const uint32_t id = c.id;
        double e = E;
        for (int l = 0; l < c.level; ++l) e = e / 2;
        out->edge[id] = e;
        out->min_x[id] = c.mnx;
        out->min_y[id] = c.mny;
        out->min_z[id] = c.mnz;
        for (int o = 0; o < 8; ++o) out->octants[(size_t)o * cap + id] = 0;
        if (c.X == NB_NONE) {
            out->body_of_node[id] = h.n;
            out->node_is_leaf[id] = 1;
            out->sum_masses[id] = 0;
            out->com_x[id] = out->com_y[id] = out->com_z[id] = 0;
            out->body_count[id] = 0;
            continue;
        }
        const uint32_t X = c.X;
        out->sum_masses[id] = h.mass[X];
        out->com_x[id] = h.comx[X];
        out->com_y[id] = h.comy[X];
        out->com_z[id] = h.comz[X];
        out->body_count[id] = h.count[X];
        if (h.body[X] != NB_NONE) {
            out->body_of_node[id] = h.body[X];
            out->node_is_leaf[id] = 1;
            continue;
        }
        out->body_of_node[id] = h.n;
        out->node_is_leaf[id] = 0;
        const uint32_t first = next_free;
        next_free += 8;
        const double ce = e / 2;
        const bool chain = c.level < (int)h.level[X];
        const uint32_t chain_oct = chain ? nb_octant_of_visit(digit_at(h, h.first[X], c.level)) : 0;
        for (uint32_t k = 0; k < 8; ++k) {
            const uint32_t o = slot_octant[k];
            out->octants[(size_t)o * cap + id] = first + k;
            Cell ch;
            ch.id = first + k;
            ch.level = c.level + 1;
            ch.mnx = (o & 2u) ? c.mnx + ce : c.mnx;
            ch.mny = (o & 4u) ? c.mny + ce : c.mny;
            ch.mnz = (o & 1u) ? c.mnz : c.mnz + ce;
            if (chain) ch.X = (o == chain_oct) ? X : NB_NONE;
            else ch.X = child[8 * (size_t)X + o];
            q.push_back(ch);
        }
    }
    // sortedBodiesInOrder: body leaves in octant order 0..7 at every level
    std::vector<uint32_t> stack{0};
    uint32_t rank = 0;
    while (!stack.empty()) {
        const uint32_t id = stack.back();
        stack.pop_back();
        if (out->node_is_leaf[id]) {
            if (out->body_of_node[id] != h.n) out->sorted_bodies[rank++] = out->body_of_node[id];
            continue;
        }
        for (int o = 7; o >= 0; --o) stack.push_back(out->octants[(size_t)o * cap + id]);
    }
    return NB_OK;
}

nb_status nb_bh_export_node_ranges(nb_bh_tree* t, uint32_t* first, uint32_t* count,
                                   uint32_t* level, uint32_t* body) {
    HostTree h;
    NB_TRY(fetch_tree(t, h, true));
    for (uint32_t k = 0; k < h.nodes; ++k) {
        if (first) first[k] = h.first[k];
        if (count) count[k] = h.count[k];
        if (level) level[k] = h.level[k];
        if (body) body[k] = h.body[k];
    }
    return NB_OK;
}

}  // extern "C"
