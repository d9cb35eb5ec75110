// nb_bh.cuh -- Barnes-Hut octree object shared by the build, traversal and export units.
//
// Layout in HBM (n_max bodies, at most 2*n_max - 1 nodes):
//  per body (sorted order): key0/key1 (u64, 21 octal digits each), ids (u32 body id)
//  per adjacent pair of sorted bodies ("split"): level (u8), start of its node (u32), end (u32)
//  per sorted position: mask (u64, levels of internal nodes whose range starts here), base (u32,
//    DFS index of the first node starting here)
//  per node (DFS pre-order, children in the reference's visit order 2,0,3,1,6,4,7,5):
//    level, first/last sorted position, skip (DFS index after the subtree), parent, body,
//    child count, centre-of-mass numerators and mass (FP64, the reference's sums), and the
//    traversal records rec64 (FP64 centre, mass, edge, skip, body: 48 B) and rec32 (FP32 centre
//    relative to the box centre, G*mass, edge^2, skip, body: 32 B).
#pragma once
#include "nb_internal.cuh"

constexpr uint32_t NB_NONE = 0xffffffffu;
constexpr int NB_KEY_LEVELS = 21;  // octal digits per 64-bit key word (bits 62..0)

struct __align__(16) NodeRec64 {
    double cx, cy, cz, mass;
    double edge;
    uint32_t skip, body;  // body = NB_NONE for internal nodes
};

struct __align__(16) NodeRec32 {
    float cx, cy, cz, gm;  // centre relative to the box centre, G * mass
    float edge2;           // edge^2
    uint32_t skip, body, level;
};

// Extra per-node data of the learned opening policy.
struct __align__(16) NodeAux {
    float spread_rel;  // mass-weighted rms distance of the cell's bodies from its centre of
                       // mass, over the cell's edge
    uint32_t count;    // bodies in the cell
    uint32_t first;    // first sorted position of the cell's bodies (they are contiguous)
    float lg_gm;       // log2(max(G * mass, 1e-37))
};

struct nb_bh_tree {
    uint32_t n_max = 0;
    uint32_t n = 0;
    uint32_t node_cap = 0;
    nb_bh_params params{};
    bool built = false;
    double G = 0;
    int device = 0;

    double* box = nullptr;  // [0..6] AABB (min xyz, max xyz, edge), [7..9] box centre
    uint32_t* info = nullptr;  // [0] node count (copy of base[n])
    uint2* tier_cells[2] = {};      // centre-of-mass tiers: cells passed up, (node, level)
    uint32_t* tier_count[2] = {};   // their count per chunk
    uint32_t* work = nullptr;  // work counter of persistent traversal kernels
    // group schedule of the learned traversal: each launch records a cost per group of 32
    // bodies, from which the next launch takes its costliest groups first
    uint32_t* group_cost = nullptr;   // per group
    uint32_t* group_first = nullptr;  // the groups taken first (priority list)
    uint32_t* group_skip = nullptr;   // bit per group: on the priority list
    uint32_t* sched = nullptr;  // [0] groups the schedule is for, [1] length of the priority
                                // list, [18..19] total cost (uint64)
    // per-body walk lengths of the last per-body FP64 traversal (accepted cells, by body id) and
    // the walk order the next one takes from them; walk_n = bodies they were recorded for (0: none)
    uint32_t* walk_len = nullptr;
    uint32_t* walk_ids = nullptr;
    mutable uint32_t walk_n = 0;
    cudaEvent_t phase_ev[6] = {};  // build phase boundaries (nb_bh_set_phase_timing)
    bool phase_timing = false;
    uint32_t records = NB_REC_ALL;   // record sets the next build computes (nb_bh_set_records)
    uint32_t built_records = 0;      // record sets of the last build

    uint64_t *key0 = nullptr, *key1 = nullptr, *key_alt = nullptr;
    uint32_t *ids = nullptr, *ids_alt = nullptr;
    uint8_t* split_level = nullptr;
    uint32_t *split_start = nullptr, *split_end = nullptr;
    uint64_t* mask = nullptr;
    uint32_t *cnt = nullptr, *base = nullptr;
    void* sort_temp = nullptr;
    uint32_t* scan_temp = nullptr;

    uint8_t* node_level = nullptr;
    uint32_t *node_first = nullptr, *node_last = nullptr, *node_skip = nullptr;
    uint32_t *node_parent = nullptr, *node_body = nullptr;
    uint32_t* node_count = nullptr;
    double *node_comx = nullptr, *node_comy = nullptr, *node_comz = nullptr, *node_mass = nullptr;
    NodeRec64* rec64 = nullptr;
    NodeRec32* rec32 = nullptr;
    float4* rec32lo = nullptr;   // second FP32 terms of rec32's centre and G*mass
    float4* rec32lo2 = nullptr;  // third FP32 terms of the centre (triple-float: exact FP64)
    double* node_q = nullptr;  // sum of m |x - box centre|^2 (for the spread)
    NodeAux* aux = nullptr;
    uint32_t* children = nullptr;  // 8 per node: children in visit order, NB_NONE padded
    float4* sorted4 = nullptr;     // per sorted position: position relative to the box centre, G*m
    float4* sorted4lo = nullptr;   // per sorted position: FP32 residual of that position (x, y, z)
    // learned opening policy (device parameters, see nb_learned.cu)
    const float* policy = nullptr;  // nullptr after nb_bh_set_policy: theta rule, same walk
    bool policy_set = false;
    uint32_t policy_flags = 0;
    float policy_log_tau = 0.f;
    float policy_theta = 0.5f;
    uint32_t policy_count_cap = 8192;
};

// NB_OK when the last build computed the record sets `need` (NB_REC_*), else an error naming
// `what`.
inline nb_status nb_need_records(const nb_bh_tree* t, uint32_t need, const char* what) {
    if ((t->built_records & need) == need) return NB_OK;
    return nb::set_error(NB_ERR_INVALID_ARG,
                         "%s: the tree was built without the node records it needs (records "
                         "0x%x built, 0x%x needed; nb_bh_set_records)",
                         what, t->built_records, need);
}

// Digit maps between the reference's octant index o = 4*(y>mid) + 2*(x>mid) + (z<mid) and the
// visit rank t (the reference pushes children 5,7,4,6,1,3,0,2 and pops 2,0,3,1,6,4,7,5).
__host__ __device__ __forceinline__ uint32_t nb_visit_of_octant(uint32_t o) {
    return (o & 4u) | ((o & 1u) << 1) | (((o >> 1) & 1u) ^ 1u);
}
__host__ __device__ __forceinline__ uint32_t nb_octant_of_visit(uint32_t t) {
    return (t & 4u) | ((t & 2u) >> 1) | (((~t) & 1u) << 1);
}
