// nb_naive.cu -- naive all-pairs acceleration (NaiveAlgorithm.cpp:262-482 semantics).
//
// Three arithmetic modes:
//  * NB_F64_IEEE: one thread per target body walks all sources j = 0..N-1 in order, every
//    operation separately rounded in the reference's order (r^2 summed left to right, den^3 as
//    (den*den)*den, 1/sqrt for rsqrt, acc += m*(r*den), G last). Bit-identical to the host
//    FP64 evaluation of NaiveAlgorithm.cpp:331-351.
//  * NB_F64: over all bodies of a large system, the FP64 form of the symmetric pair kernel of
//    nb_pair_sym.cu (each unordered pair once, 20 FP64 operations for both bodies); otherwise the
//    same loop as the IEEE mode with FMAs and m (r^2 + eps^2)^(-3/2) from the hardware rsqrt
//    estimate with one correction (nb_m_rinv3_f64; FP64-pipe bound on GB300).
//  * NB_F32C: over all bodies of a large system, the symmetric FP32 pair kernel of
//    nb_pair_sym.cu (each unordered pair once, added to both bodies); otherwise (target ranges,
//    small systems) the one-sided FP32-compensated pair kernel of nb_pair.cuh (scalar FP32 pair
//    math, TwoSum accumulation, stream-K persistent CTAs, cp.async.bulk j-tiles behind bounded
//    mbarrier waits), run as a batch of one system.
//  * NB_DF64: double-float pair math on the FP32 pipe (FP64-accurate to ~1e-14); over all bodies
//    of a large system the double-float form of the symmetric pair kernel.
#include "nb_internal.cuh"
#include "nb_pair.cuh"
#include "nb_pair_sym.cuh"

namespace {

// ---------------------------------------------------------------------------------------------
// FP64
// ---------------------------------------------------------------------------------------------
constexpr int F64_THREADS = 64;

// blockIdx.y selects a chunk of `chunk` sources (NB_F64 at small n, for more warps per SM; the
// IEEE mode always runs one chunk so that its sum order stays the reference's); with more than
// one chunk the partial sums (times G) go to part[(chunk index * n_t + target) * 3 + axis].
template <bool IEEE>
__global__ void __launch_bounds__(F64_THREADS)
naive_f64_kernel(const double* __restrict__ m, const double* __restrict__ x,
                 const double* __restrict__ y, const double* __restrict__ z,
                 double* __restrict__ ax, double* __restrict__ ay, double* __restrict__ az,
                 uint32_t n, uint32_t i_begin, uint32_t i_end, double G, double eps2,
                 uint32_t chunk, double* __restrict__ part) {
    __shared__ double sx[F64_THREADS], sy[F64_THREADS], sz[F64_THREADS], sm[F64_THREADS];
    const uint32_t i = i_begin + blockIdx.x * F64_THREADS + threadIdx.x;
    const bool active = i < i_end;
    double px = 0, py = 0, pz = 0;
    if (active) {
        px = x[i];
        py = y[i];
        pz = z[i];
    }
    double acc_x = 0, acc_y = 0, acc_z = 0;
    const uint32_t j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    for (uint32_t k = j0; k < j1; k += F64_THREADS) {
        const uint32_t j = k + threadIdx.x;
        if (j < j1) {
            sx[threadIdx.x] = x[j];
            sy[threadIdx.x] = y[j];
            sz[threadIdx.x] = z[j];
            sm[threadIdx.x] = m[j];
        }
        __syncthreads();
        const uint32_t cnt = min((uint32_t)F64_THREADS, j1 - k);
        if (active) {
            if (IEEE) {
                for (uint32_t jj = 0; jj < cnt; ++jj) {
                    const double r_x = __dsub_rn(sx[jj], px);
                    const double r_y = __dsub_rn(sy[jj], py);
                    const double r_z = __dsub_rn(sz[jj], pz);
                    double den = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(r_x, r_x), __dmul_rn(r_y, r_y)),
                                                     __dmul_rn(r_z, r_z)),
                                           eps2);
                    den = __dmul_rn(__dmul_rn(den, den), den);
                    den = __ddiv_rn(1.0, __dsqrt_rn(den));
                    acc_x = __dadd_rn(acc_x, __dmul_rn(sm[jj], __dmul_rn(r_x, den)));
                    acc_y = __dadd_rn(acc_y, __dmul_rn(sm[jj], __dmul_rn(r_y, den)));
                    acc_z = __dadd_rn(acc_z, __dmul_rn(sm[jj], __dmul_rn(r_z, den)));
                }
            } else {
#pragma unroll 4
                for (uint32_t jj = 0; jj < cnt; ++jj) {
                    const double r_x = sx[jj] - px;
                    const double r_y = sy[jj] - py;
                    const double r_z = sz[jj] - pz;
                    const double den = fma(r_x, r_x, fma(r_y, r_y, fma(r_z, r_z, eps2)));
                    const double s = nb_m_rinv3_f64(sm[jj], den);
                    acc_x = fma(s, r_x, acc_x);
                    acc_y = fma(s, r_y, acc_y);
                    acc_z = fma(s, r_z, acc_z);
                }
            }
        }
        __syncthreads();
    }
    if (active) {
        if (IEEE) {
            ax[i] = __dmul_rn(acc_x, G);
            ay[i] = __dmul_rn(acc_y, G);
            az[i] = __dmul_rn(acc_z, G);
        } else if (gridDim.y == 1) {
            ax[i] = acc_x * G;
            ay[i] = acc_y * G;
            az[i] = acc_z * G;
        } else {
            double* o = part + ((size_t)blockIdx.y * (i_end - i_begin) + (i - i_begin)) * 3;
            o[0] = acc_x * G;
            o[1] = acc_y * G;
            o[2] = acc_z * G;
        }
    }
}

// Adds the chunks' partial sums of each target in chunk order.
__global__ void chunk_combine_kernel(const double* __restrict__ part, uint32_t chunks,
                                  uint32_t i_begin, uint32_t i_end, double* __restrict__ ax,
                                  double* __restrict__ ay, double* __restrict__ az) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n_t = i_end - i_begin;
    if (t >= n_t) return;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (uint32_t c = 0; c < chunks; ++c) {
        const double* o = part + ((size_t)c * n_t + t) * 3;
        sx += o[0];
        sy += o[1];
        sz += o[2];
    }
    ax[i_begin + t] = sx;
    ay[i_begin + t] = sy;
    az[i_begin + t] = sz;
}

// Number and size (a multiple of `tile`) of the source chunks that give at least ~8 warps per SM
// when blocks_per_chunk blocks cover the targets.
void choose_chunks(const nb_ctx* ctx, int blocks_per_chunk, uint32_t n, uint32_t tile,
                   uint32_t* chunks, uint32_t* chunk) {
    uint32_t c = (uint32_t)nb::ceil_div(8LL * ctx->sm_count, blocks_per_chunk);
    c = min(c, 32u);
    c = min(c, (uint32_t)nb::ceil_div(n, tile));
    if (c < 1) c = 1;
    *chunk = (uint32_t)nb::ceil_div(nb::ceil_div(n, c), tile) * tile;
    *chunks = (uint32_t)nb::ceil_div(n, *chunk);
}

// FP64 accelerations of listed target bodies (ax[t] for targets[t]); FMAs + refined rsqrt.
__global__ void __launch_bounds__(F64_THREADS)
naive_f64_targets_kernel(const double* __restrict__ m, const double* __restrict__ x,
                         const double* __restrict__ y, const double* __restrict__ z, uint32_t n,
                         const uint32_t* __restrict__ targets, uint32_t n_t,
                         double* __restrict__ ax, double* __restrict__ ay,
                         double* __restrict__ az, double G, double eps2) {
    __shared__ double sx[F64_THREADS], sy[F64_THREADS], sz[F64_THREADS], sm[F64_THREADS];
    const uint32_t t = blockIdx.x * F64_THREADS + threadIdx.x;
    const bool active = t < n_t;
    const uint32_t i = active ? targets[t] : 0;
    const double px = active ? x[i] : 0, py = active ? y[i] : 0, pz = active ? z[i] : 0;
    double acc_x = 0, acc_y = 0, acc_z = 0;
    for (uint32_t k = 0; k < n; k += F64_THREADS) {
        const uint32_t j = k + threadIdx.x;
        if (j < n) {
            sx[threadIdx.x] = x[j];
            sy[threadIdx.x] = y[j];
            sz[threadIdx.x] = z[j];
            sm[threadIdx.x] = m[j];
        }
        __syncthreads();
        const uint32_t cnt = min((uint32_t)F64_THREADS, n - k);
        if (active) {
#pragma unroll 4
            for (uint32_t jj = 0; jj < cnt; ++jj) {
                const double r_x = sx[jj] - px, r_y = sy[jj] - py, r_z = sz[jj] - pz;
                const double den = fma(r_x, r_x, fma(r_y, r_y, fma(r_z, r_z, eps2)));
                const double s = nb_m_rinv3_f64(sm[jj], den);
                acc_x = fma(s, r_x, acc_x);
                acc_y = fma(s, r_y, acc_y);
                acc_z = fma(s, r_z, acc_z);
            }
        }
        __syncthreads();
    }
    if (active) {
        ax[t] = acc_x * G;
        ay[t] = acc_y * G;
        az[t] = acc_z * G;
    }
}

// ---------------------------------------------------------------------------------------------
// FP32, compensated: the batched pair kernel (nb_pair.cuh) with a batch of one system whose
// targets are [i_begin, i_end).
// ---------------------------------------------------------------------------------------------
int g_naive_pair_cfg = 0;  // tile configuration (nb_naive_set_pair_config)
// Symmetric kernel (nb_pair_sym.cu) for full target ranges (nb_naive_set_symmetric): mode 0
// never, 1 automatic, 2 always; and its FP32, FP64 and double-float shapes.
int g_naive_sym_mode = 1;
int g_naive_sym_cfg[3] = {0, 0, 0};
// Automatic selection wants at least this many units per persistent CTA (the one-sided kernels
// spread small systems better) and j-side partials (3 values per unit and tile body) below the
// cap. With 7, a 16,384-body system takes the FP64 shape (4,2,64) at its 7 resident CTAs per SM
// (8,320 units over 1,064 CTAs) and the larger (4,4,64) I-block from ~18,000 bodies on.
constexpr uint64_t SYM_MIN_UNITS_PER_CTA = 7;
constexpr size_t SYM_PART_CAP_BYTES = (size_t)4 << 30;

// Runs the symmetric kernel of arithmetic form `form` (nb::SymForm) for the whole system when
// the mode and the plan allow it; *done tells whether it did.
nb_status naive_sym(nb_ctx* ctx, int form, const double* m, const double* x, const double* y,
                    const double* z, double* ax, double* ay, double* az, uint32_t n, double G,
                    double eps2, cudaStream_t stream, bool* done) {
    *done = false;
    if (g_naive_sym_mode == 0) return NB_OK;
    // candidate shapes: the configured one, except in the automatic mode of the FP64 and
    // double-float forms, where shape 1 is (4,4,64) with 512-body I-blocks and shape 0 (4,2,64)
    // with 256: FP64 prefers the larger I-block (same speed, half the partials: 24 bytes per
    // unit and tile body), double-float the smaller one (faster: fewer registers per thread)
    int cand[2] = {g_naive_sym_cfg[form], -1};
    if (g_naive_sym_mode == 1 && form == nb::SYM_F64) {
        cand[0] = 1;
        cand[1] = 0;
    } else if (g_naive_sym_mode == 1 && form == nb::SYM_DF) {
        cand[0] = 0;
        cand[1] = 1;
    }
    int cfg = -1;
    nb::SymHostPlan hp;
    size_t pj_bytes = 0;
    for (int c : cand) {
        if (c < 0) break;
        NB_TRY(nb::sym_host_plan(form, c, &n, 1, ctx->sm_count, &hp));
        pj_bytes = nb::sym_part_j_bytes(form, c, hp.units);
        if (g_naive_sym_mode == 2 || (hp.units >= SYM_MIN_UNITS_PER_CTA * hp.ctas &&
                                      pj_bytes <= SYM_PART_CAP_BYTES)) {
            cfg = c;
            break;
        }
    }
    if (cfg < 0) return NB_OK;
    auto al = [](size_t v) { return (v + 255) & ~(size_t)255; };
    const size_t table_bytes = al(2 * sizeof(nbsym::SymSys));
    const size_t src_bytes = al((size_t)hp.n_records * nb::sym_record_bytes(form));
    const size_t pi_bytes = al(nb::sym_part_i_bytes(form, cfg, hp.ctas, hp.n_blocks));
    void* base = nullptr;
    NB_TRY(nb::scratch(ctx, NB_SCRATCH_PAIR_SYM, table_bytes + src_bytes + pi_bytes + pj_bytes,
                       &base));
    char* b = (char*)base;
    nbsym::SymSys* table = (nbsym::SymSys*)b;
    NB_TRY(nb::sym_single_table(table, hp, stream));
    nbsym::SymPlan S;
    S.sys = table;
    S.n_systems = 1;
    S.ctas = hp.ctas;
    S.n_total = hp.n_total;
    S.n_records = hp.n_records;
    S.units = hp.units;
    S.wait_limit = ctx->wait_limit;
    b += table_bytes;
    *done = true;
    return nb::sym_launch(form, cfg, S, m, x, y, z, G, eps2, b, b + src_bytes,
                          b + src_bytes + pi_bytes, ax, ay, az, ctx->dev_error, stream);
}

nb_status naive_f32c(nb_ctx* ctx, const double* m, const double* x, const double* y,
                     const double* z, double* ax, double* ay, double* az, uint32_t n,
                     uint32_t i_begin, uint32_t i_end, double G, double eps2,
                     cudaStream_t stream) {
    if (i_begin == 0 && i_end == n) {
        bool done = false;
        NB_TRY(naive_sym(ctx, nb::SYM_F32, m, x, y, z, ax, ay, az, n, G, eps2, stream, &done));
        if (done) return NB_OK;
    }
    const int cfg = g_naive_pair_cfg;
    const nb::PairConfig& C = nb::kPairConfigs[cfg];
    int per_sm = 0;
    NB_TRY(nb::pair_ctas_per_sm(cfg, &per_sm));
    const uint32_t n_t = i_end - i_begin;
    const uint32_t ib = (uint32_t)(C.threads * C.ip);
    const uint32_t n_ib = (n_t + ib - 1) / ib;
    const uint32_t n_jt = (n + C.jt - 1) / C.jt;
    const uint64_t units = (uint64_t)n_ib * n_jt;
    uint64_t ctas = (uint64_t)ctx->sm_count * per_sm;
    if (ctas > units) ctas = units;
    // scratch: plan arrays, duplicated sources, float4 targets, partials
    const size_t plan_bytes = 512;
    const size_t src_bytes = ((size_t)n * sizeof(nbpair::SrcDup) + 255) & ~(size_t)255;
    const size_t tgt_bytes = ((size_t)n * sizeof(float4) + 255) & ~(size_t)255;
    const size_t part_bytes = nb::pair_partial_floats(cfg, (uint32_t)ctas, n_ib) * sizeof(float);
    void* base = nullptr;
    NB_TRY(nb::scratch(ctx, NB_SCRATCH_NAIVE_F32, plan_bytes + src_bytes + tgt_bytes + part_bytes,
                       &base));
    char* b = (char*)base;
    uint64_t* unit_off = (uint64_t*)b;
    uint32_t* sys_off = (uint32_t*)(b + 64);
    uint32_t* tgt_begin = (uint32_t*)(b + 128);
    uint32_t* t_off = (uint32_t*)(b + 192);
    uint32_t* ib_off = (uint32_t*)(b + 256);
    nbpair::SrcDup* src = (nbpair::SrcDup*)(b + plan_bytes);
    float4* tgt = (float4*)(b + plan_bytes + src_bytes);
    float* part = (float*)(b + plan_bytes + src_bytes + tgt_bytes);
    NB_TRY(nb::pair_plan_single(sys_off, tgt_begin, t_off, unit_off, ib_off, n, i_begin, i_end,
                                units, n_ib, stream));
    nbpair::Plan P;
    P.n_systems = 1;
    P.ctas = (uint32_t)ctas;
    P.units = units;
    P.sys_off = sys_off;
    P.tgt_begin = tgt_begin;
    P.t_off = t_off;
    P.unit_off = unit_off;
    P.ib_off = ib_off;
    P.wait_limit = ctx->wait_limit;
    return nb::pair_launch(cfg, P, m, x, y, z, n, n_t, G, eps2, src, tgt, part, ax, ay, az,
                           ctx->dev_error, stream);
}

// ---------------------------------------------------------------------------------------------
// Double-float (NB_DF64): FP64-accurate pair math on the FP32 pipe
// ---------------------------------------------------------------------------------------------
constexpr int DF_THREADS = 128;
constexpr int DF_TILE = 128;

// Source record: the position minus body 0 (exact) as triple-floats and G*m as a double-float.
struct __align__(16) SrcTF {
    float xh, xm, xl, yh, ym, yl, zh, zm, zl, gh, gl, pad;
};

__global__ void df_prepare_kernel(const double* __restrict__ m, const double* __restrict__ x,
                                  const double* __restrict__ y, const double* __restrict__ z,
                                  uint32_t n, double G, SrcTF* __restrict__ out) {
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    SrcTF r;
    tf_split_diff(x[b], x[0], r.xh, r.xm, r.xl);
    tf_split_diff(y[b], y[0], r.yh, r.ym, r.yl);
    tf_split_diff(z[b], z[0], r.zh, r.zm, r.zl);
    const double gm = G * m[b];
    r.gh = (float)gm;
    r.gl = (float)(gm - (double)r.gh);
    r.pad = 0.f;
    out[b] = r;
}

// One thread per target; sources in shared-memory tiles. Per pair: exact separations from the
// triple-floats, r^2 + eps^2 with TwoSums, 1/r from the hardware estimate with an error-free
// correction, G m / r^3 and the products in double-float (the same arithmetic as the
// Barnes-Hut double-float monopole), Neumaier-compensated sums per tile added into FP64. The
// self pair contributes exactly 0.
// blockIdx.y selects a chunk of `chunk` sources; with more than one chunk the partial sums go
// to part[(chunk index * n_t + target) * 3 + axis] and df_combine_kernel adds them in order.
__global__ void __launch_bounds__(DF_THREADS)
naive_df_kernel(const SrcTF* __restrict__ src, uint32_t n, uint32_t i_begin, uint32_t i_end,
                uint32_t chunk, float e2h, float e2l, double* __restrict__ ax,
                double* __restrict__ ay, double* __restrict__ az, double* __restrict__ part) {
    __shared__ SrcTF tile[DF_TILE];
    const uint32_t i = i_begin + blockIdx.x * DF_THREADS + threadIdx.x;
    const bool active = i < i_end;
    SrcTF me{};
    if (active) me = src[i];
    double sum_x = 0.0, sum_y = 0.0, sum_z = 0.0;
    const uint32_t j0 = blockIdx.y * chunk, j1 = min(n, j0 + chunk);
    for (uint32_t k = j0; k < j1; k += DF_TILE) {
        float ahx = 0.f, ahy = 0.f, ahz = 0.f, alx = 0.f, aly = 0.f, alz = 0.f;
        for (uint32_t j = threadIdx.x; j < DF_TILE && k + j < j1; j += DF_THREADS)
            tile[j] = src[k + j];
        __syncthreads();
        const uint32_t cnt = min((uint32_t)DF_TILE, j1 - k);
        if (active) {
            for (uint32_t jj = 0; jj < cnt; ++jj) {
                const SrcTF c = tile[jj];
                const nb_df dx = tf_diff(c.xh, c.xm, c.xl, me.xh, me.xm, me.xl);
                const nb_df dy = tf_diff(c.yh, c.ym, c.yl, me.yh, me.ym, me.yl);
                const nb_df dz = tf_diff(c.zh, c.zm, c.zl, me.zh, me.zm, me.zl);
                const nb_df sx = df_sqr(dx), sy = df_sqr(dy), sz = df_sqr(dz);
                nb_df a = df_two_sum(sx.h, sy.h);
                a.l += sx.l + sy.l;
                nb_df b = df_two_sum(a.h, sz.h);
                b.l += a.l + sz.l;
                nb_df e = df_two_sum(b.h, e2h);
                e.l += b.l + e2l;
                const nb_df r2 = df_two_sum(e.h, e.l);
                const float y0 = nb_rsqrt_f32(r2.h);
                const float q = y0 * y0, qe = fmaf(y0, y0, -q);
                const float th = r2.h * q;
                float te = fmaf(r2.h, q, -th);
                te = fmaf(r2.h, qe, te);
                te = fmaf(r2.l, q, te);
                const float ee = (1.0f - th) - te;
                const nb_df inv = df_fast_two_sum(y0, y0 * (ee * fmaf(0.375f, ee, 0.5f)));
                const nb_df w = df_mul(nb_df{c.gh, c.gl}, df_mul(df_sqr(inv), inv));
                const nb_df tx = df_mul(dx, w), ty = df_mul(dy, w), tz = df_mul(dz, w);
                nb_df t = df_two_sum(ahx, tx.h);
                ahx = t.h;
                alx += t.l + tx.l;
                t = df_two_sum(ahy, ty.h);
                ahy = t.h;
                aly += t.l + ty.l;
                t = df_two_sum(ahz, tz.h);
                ahz = t.h;
                alz += t.l + tz.l;
            }
            // the tile's compensated sum into FP64 (3 FP64 adds per tile): the FP32 low part
            // of a compensated sum over all n terms would lose digits at large n
            sum_x += (double)ahx + (double)alx;
            sum_y += (double)ahy + (double)aly;
            sum_z += (double)ahz + (double)alz;
        }
        __syncthreads();
    }
    if (!active) return;
    if (gridDim.y == 1) {
        ax[i] = sum_x;
        ay[i] = sum_y;
        az[i] = sum_z;
    } else {
        double* o = part + ((size_t)blockIdx.y * (i_end - i_begin) + (i - i_begin)) * 3;
        o[0] = sum_x;
        o[1] = sum_y;
        o[2] = sum_z;
    }
}


nb_status naive_df64(nb_ctx* ctx, const double* m, const double* x, const double* y,
                     const double* z, double* ax, double* ay, double* az, uint32_t n,
                     uint32_t i_begin, uint32_t i_end, double G, double eps2,
                     cudaStream_t stream) {
    // split the sources into chunks when the targets alone give too few warps per SM
    const uint32_t n_t = i_end - i_begin;
    const int blocks = nb::ceil_div(n_t, DF_THREADS);
    uint32_t chunks = 1, chunk = n;
    choose_chunks(ctx, blocks, n, DF_TILE, &chunks, &chunk);
    const size_t src_bytes = ((size_t)n * sizeof(SrcTF) + 255) & ~(size_t)255;
    const size_t part_bytes = chunks > 1 ? (size_t)chunks * n_t * 3 * sizeof(double) : 0;
    void* base = nullptr;
    NB_TRY(nb::scratch(ctx, NB_SCRATCH_NAIVE_DF, src_bytes + part_bytes, &base));
    SrcTF* src = (SrcTF*)base;
    double* part = (double*)((char*)base + src_bytes);
    df_prepare_kernel<<<nb::ceil_div(n, 256), 256, 0, stream>>>(m, x, y, z, n, G, src);
    NB_TRY(nb::check_launch("df_prepare_kernel"));
    const float e2h = (float)eps2, e2l = (float)(eps2 - (double)e2h);
    naive_df_kernel<<<dim3(blocks, chunks), DF_THREADS, 0, stream>>>(
        src, n, i_begin, i_end, chunk, e2h, e2l, ax, ay, az, part);
    NB_TRY(nb::check_launch("naive_df_kernel"));
    if (chunks == 1) return NB_OK;
    chunk_combine_kernel<<<nb::ceil_div(n_t, 256), 256, 0, stream>>>(part, chunks, i_begin,
                                                                     i_end, ax, ay, az);
    return nb::check_launch("chunk_combine_kernel");
}

nb_status naive_dispatch(nb_ctx* ctx, const double* m, const double* x, const double* y,
                         const double* z, double* ax, double* ay, double* az, uint32_t n,
                         uint32_t i_begin, uint32_t i_end, double G, double eps2,
                         nb_precision prec, cudaStream_t stream) {
    NB_CHECK_CTX(ctx);
    if (n == 0 || i_begin >= i_end) return NB_OK;
    if (!m || !x || !y || !z || !ax || !ay || !az)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_accel: null array pointer");
    if (i_end > n) return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_accel: i_end > n");
    const uint32_t n_t = i_end - i_begin;
    switch (prec) {
        case NB_F64_IEEE:
            naive_f64_kernel<true><<<nb::ceil_div(n_t, F64_THREADS), F64_THREADS, 0, stream>>>(
                m, x, y, z, ax, ay, az, n, i_begin, i_end, G, eps2, n, nullptr);
            return nb::check_launch("naive_f64_kernel<ieee>");
        case NB_F64: {
            if (i_begin == 0 && i_end == n) {
                bool done = false;
                NB_TRY(naive_sym(ctx, nb::SYM_F64, m, x, y, z, ax, ay, az, n, G, eps2, stream,
                                 &done));
                if (done) return NB_OK;
            }
            const int blocks = nb::ceil_div(n_t, F64_THREADS);
            uint32_t chunks = 1, chunk = n;
            choose_chunks(ctx, blocks, n, F64_THREADS, &chunks, &chunk);
            double* part = nullptr;
            if (chunks > 1) {
                void* base = nullptr;
                NB_TRY(nb::scratch(ctx, NB_SCRATCH_NAIVE_DF, (size_t)chunks * n_t * 3 * 8, &base));
                part = (double*)base;
            }
            naive_f64_kernel<false><<<dim3(blocks, chunks), F64_THREADS, 0, stream>>>(
                m, x, y, z, ax, ay, az, n, i_begin, i_end, G, eps2, chunk, part);
            NB_TRY(nb::check_launch("naive_f64_kernel"));
            if (chunks == 1) return NB_OK;
            chunk_combine_kernel<<<nb::ceil_div(n_t, 256), 256, 0, stream>>>(part, chunks, i_begin,
                                                                             i_end, ax, ay, az);
            return nb::check_launch("chunk_combine_kernel");
        }
        case NB_F32C:
            return naive_f32c(ctx, m, x, y, z, ax, ay, az, n, i_begin, i_end, G, eps2, stream);
        case NB_DF64: {
            if (i_begin == 0 && i_end == n) {
                bool done = false;
                NB_TRY(naive_sym(ctx, nb::SYM_DF, m, x, y, z, ax, ay, az, n, G, eps2, stream,
                                 &done));
                if (done) return NB_OK;
            }
            return naive_df64(ctx, m, x, y, z, ax, ay, az, n, i_begin, i_end, G, eps2, stream);
        }
        default:
            return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_accel: unknown precision %d",
                                 (int)prec);
    }
}

}  // namespace

extern "C" {

nb_status nb_naive_accel(nb_ctx* ctx, const double* m, const double* x, const double* y,
                         const double* z, double* ax, double* ay, double* az, uint32_t n,
                         double G, double eps2, nb_precision prec, int block_size,
                         nb_stream_t stream) {
    if (block_size < 0)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_accel: block_size must be >= 0");
    return naive_dispatch(ctx, m, x, y, z, ax, ay, az, n, 0, n, G, eps2, prec,
                          (cudaStream_t)stream);
}

nb_status nb_naive_accel_targets(nb_ctx* ctx, const double* m, const double* x, const double* y,
                                 const double* z, uint32_t n, const uint32_t* targets,
                                 uint32_t n_targets, double* ax, double* ay, double* az, double G,
                                 double eps2, nb_stream_t stream) {
    NB_CHECK_CTX(ctx);
    if (!m || !x || !y || !z || !targets || !ax || !ay || !az)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_accel_targets: null pointer");
    if (n == 0 || n_targets == 0) return NB_OK;
    naive_f64_targets_kernel<<<nb::ceil_div(n_targets, F64_THREADS), F64_THREADS, 0,
                               (cudaStream_t)stream>>>(m, x, y, z, n, targets, n_targets, ax, ay,
                                                       az, G, eps2);
    return nb::check_launch("naive_f64_targets_kernel");
}

nb_status nb_naive_set_pair_config(int config) {
    if (config < 0 || config >= nb::NB_PAIR_CONFIGS)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_set_pair_config: config %d", config);
    g_naive_pair_cfg = config;
    return NB_OK;
}

nb_status nb_naive_set_symmetric(int mode, int config_f32, int config_f64, int config_df) {
    if (mode < 0 || mode > 2)
        return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_set_symmetric: mode %d", mode);
    const int cfg[3] = {config_f32, config_f64, config_df};
    for (int f = 0; f < 3; ++f)
        if (cfg[f] < 0 || cfg[f] >= nb::sym_config_count(f))
            return nb::set_error(NB_ERR_INVALID_ARG, "nb_naive_set_symmetric: config %d of form %d",
                                 cfg[f], f);
    g_naive_sym_mode = mode;
    for (int f = 0; f < 3; ++f) g_naive_sym_cfg[f] = cfg[f];
    return NB_OK;
}

nb_status nb_naive_accel_range(nb_ctx* ctx, const double* m, const double* x, const double* y,
                               const double* z, double* ax, double* ay, double* az, uint32_t n,
                               uint32_t i_begin, uint32_t i_end, double G, double eps2,
                               nb_precision prec, nb_stream_t stream) {
    return naive_dispatch(ctx, m, x, y, z, ax, ay, az, n, i_begin, i_end, G, eps2, prec,
                          (cudaStream_t)stream);
}

}  // extern "C"
