// gpp_gemm_mixed.cu -- unoccupied bands with band-independent frequencies in
// mixed precision: the band sum G = sum_n1 c aqsn as a float-float complex
// GEMM on the FP32 pipes, then the frequency pass on G (the FP64 form of the
// same factorisation, and its derivation, is gpp_gemm.cu).
//
// The GEMM keeps the packed layout of the mixed kernels: a thread owns one
// G' row pair -- the two lanes of every f32x2 instruction -- and 8 columns.
// Complex products take Gauss's 3M form with three float-float accumulators
// per output (ar br, ai bi, (ar + ai)(br + bi)), so one complex multiply-add
// of both rows is 36 packed instructions (3 products, 3 TwoSum-based
// additions) instead of 48; the sums re + im are formed once per staged
// element.  A block computes 8 row pairs x 128 columns, staging 8 bands of
// c and aqsn per step in shared memory.  G is written as row-pair planes like
// wtilde and Q, and the frequency pass reads it exactly as the per-term
// kernel reads aqsn * Q:
// terms within 1e-3 |wx| of the pole are recomputed in FP64 from the inputs
// and G.  Compared with the per-term kernel the division runs once per
// (row, column, frequency) instead of once per band.  The per-band output
// acht_n1_loc is a second product of the same form, H = aqsn M_2^T, with
// its long sum over columns split into chunks that are added in order.
#include "gpp_gemm_mixed.h"
#include "gpp_ozaki_split.cuh"
#include "gpp_tiles_mixed.cuh"

namespace gpp {

gpp_status set_error(gpp_status s, const char *msg);

namespace {

constexpr int kThreads = 256;
// The two float-float GEMMs: 128 threads, 8 row pairs per block, so 16
// threads per row pair, each owning kPerThread columns (G) or bands (H) with
// three df accumulators apiece; kStep k values per shared-memory step.
// Shapes and resident blocks as measured fastest on the GB300 at the
// production shape among 8 x 128 / 8 x 64 / 4 x 128 tiles at 3-5 blocks per
// SM: G 8 x 128 at 3 blocks (168 registers), H 8 x 64 at 5 (at most 102).
constexpr int kGemmThreads = 128;
constexpr int kPairs = 8;      // row pairs per GEMM block
constexpr int kLanes = kGemmThreads / kPairs;  // threads per row pair (16)
constexpr int kStep = 8;       // k values per shared-memory step
constexpr int kCols = 128;     // G: columns per block
constexpr int kGMinBlocks = 3;
constexpr int kHBands = 64;    // H: bands per block
constexpr int kHMinBlocks = 5;

size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }
int row_pairs(const Problem &p) { return (p.ng + 1) / 2; }

gpp_status cuda_fail(cudaError_t e, const char *what) {
    char buf[256];
    snprintf(buf, sizeof(buf), "%s: %s", what, cudaGetErrorString(e));
    return set_error(e == cudaErrorMemoryAllocation ? GPP_ERR_OUT_OF_MEMORY : GPP_ERR_CUDA, buf);
}

// c[k][j] = 0.5 vcoul[igp] conj(aqsm[b0 + k][igp]) for rows 2j, 2j+1 as
// float-float lanes: two float4 (re, im), each (hi r0, hi r1, lo r0, lo r1).
// A row past ngpown or with an invalid G' index contributes 0.
__global__ void __launch_bounds__(kThreads) mg_coeff_kernel(Problem p, int b0, int K,
                                                            float4 *cpl, int *err) {
    const int pairs = (p.ng + 1) / 2;
    const long long n = (long long)K * pairs;
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        const int k = (int)(i / pairs), j = (int)(i % pairs);
        df re[2], im[2];
        for (int g = 0; g < 2; ++g) {
            const int r = 2 * j + g;
            double2 c = make_double2(0.0, 0.0);
            if (r < p.ng) {
                const int igp = resolve_igp(p, r, err);
                if (igp >= 0) {
                    const double2 m = __ldg(p.aqsm + (size_t)(b0 + k) * p.nc + igp);
                    c = cscale(make_double2(0.5 * m.x, -0.5 * m.y), __ldg(p.vcoul + igp));
                }
            }
            re[g] = split_bits(c.x);
            im[g] = split_bits(c.y);
        }
        cpl[i * 2] = make_float4(re[0].h, re[1].h, re[0].l, re[1].l);
        cpl[i * 2 + 1] = make_float4(im[0].h, im[1].h, im[0].l, im[1].l);
    }
}

// One k step of the 3M (Gauss) float-float complex multiply-add for kPer
// outputs: a = ar + i ai (the row pair's lanes, sa = ar + ai) times
// b = br + i bi (broadcast, sb = br + bi).  P1 = ar br, P2 = ai bi and
// P3 = sa sb accumulate separately; the product sum is P1 - P2 + i (P3 - P1
// - P2), formed once at the end (mg_3m_result).  Three df products and three
// df sums per output and k -- 36 packed instructions, against 48 for the
// four products and four sums of the direct form.
template <int PER>
__device__ __forceinline__ void mg_3m_step(const float4 a4, const float4 b4, const float4 s4,
                                           const float4 *bv, const float2 *sv, int stride,
                                           df2 (&acc)[3][PER]) {
    const df2 ar = {f2(a4.x, a4.y), f2(a4.z, a4.w)};
    const df2 ai = {f2(b4.x, b4.y), f2(b4.z, b4.w)};
    const df2 sa = {f2(s4.x, s4.y), f2(s4.z, s4.w)};
#pragma unroll
    for (int t = 0; t < PER; ++t) {
        const float4 v = bv[t * stride];
        const float2 w = sv[t * stride];
        acc[0][t] = df2_add(acc[0][t], df2_mul(ar, df2_bcast(df{v.x, v.y})));
        acc[1][t] = df2_add(acc[1][t], df2_mul(ai, df2_bcast(df{v.z, v.w})));
        acc[2][t] = df2_add(acc[2][t], df2_mul(sa, df2_bcast(df{w.x, w.y})));
    }
}

// Real and imaginary parts from the three sums, renormalised (the
// imaginary part can cancel), as two float4 (hi r0, hi r1, lo r0, lo r1).
__device__ __forceinline__ void mg_3m_result(const df2 &p1, const df2 &p2, const df2 &p3,
                                             float4 &re, float4 &im) {
    const df2 r = df2_norm(df2_sub(p1, p2));
    const df2 i = df2_norm(df2_sub(df2_sub(p3, p1), p2));
    re = make_float4(r.h.x, r.h.y, r.l.x, r.l.y);
    im = make_float4(i.h.x, i.h.y, i.l.x, i.l.y);
}

// Staging of the 3M operands: the row pair's (re, im, re + im) and the
// broadcast operand's (re, im) float4 with its re + im as a float2; the
// sums are renormalised df values, formed once per staged element.
__device__ __forceinline__ void mg_stage_a(float4 re, float4 im, float4 *dst) {
    const df2 s = df2_norm(df2_add(df2{f2(re.x, re.y), f2(re.z, re.w)},
                                   df2{f2(im.x, im.y), f2(im.z, im.w)}));
    dst[0] = re;
    dst[1] = im;
    dst[2] = make_float4(s.h.x, s.h.y, s.l.x, s.l.y);
}
__device__ __forceinline__ void mg_stage_b(float4 v, float4 *dst, float2 *sum) {
    const df s = df_norm(df_add(df{v.x, v.y}, df{v.z, v.w}));
    *dst = v;
    *sum = make_float2(s.h, s.l);
}

// G[j][col] = sum_k c[k][j] aqsn[k][col] in float-float, both rows of pair j
// as the lanes.  Grid: x over blocks of kPairs row pairs (fastest, so blocks
// in flight share their aqsn columns in L2), y over blocks of kCols columns.
__global__ void __launch_bounds__(kGemmThreads, kGMinBlocks) mg_gemm_kernel(
    int K, int pairs, int nc, const float4 *__restrict__ cpl, const float4 *__restrict__ band,
    float4 *__restrict__ G) {
    __shared__ float4 sA[kStep][kPairs][3];
    __shared__ float4 sB[kStep][kCols];
    __shared__ float2 sS[kStep][kCols];
    constexpr int kPerThread = kCols / kLanes;
    const int tid = threadIdx.x;
    const int pr = tid / kLanes, cg = tid % kLanes;
    const int pair0 = blockIdx.x * kPairs, col0 = blockIdx.y * kCols;
    const df2 z = {f2(0.f, 0.f), f2(0.f, 0.f)};
    df2 acc[3][kPerThread];
#pragma unroll
    for (int t = 0; t < kPerThread; ++t) acc[0][t] = acc[1][t] = acc[2][t] = z;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k0 = 0; k0 < K; k0 += kStep) {
        const int kc = min(kStep, K - k0);
        __syncthreads();  // the previous step's operands are consumed
        for (int i = tid; i < kStep * kPairs; i += kGemmThreads) {
            const int kk = i / kPairs, pp = i % kPairs;
            float4 re = zero4, im = zero4;
            if (kk < kc && pair0 + pp < pairs) {
                const float4 *c = cpl + ((size_t)(k0 + kk) * pairs + pair0 + pp) * 2;
                re = c[0];
                im = c[1];
            }
            mg_stage_a(re, im, sA[kk][pp]);
        }
        for (int i = tid; i < kStep * kCols; i += kGemmThreads) {
            const int kk = i / kCols, cc = i % kCols;
            float4 v = zero4;
            if (kk < kc && col0 + cc < nc) v = band[(size_t)(k0 + kk) * nc + col0 + cc];
            mg_stage_b(v, &sB[kk][cc], &sS[kk][cc]);
        }
        __syncthreads();
        for (int kk = 0; kk < kc; ++kk)
            mg_3m_step<kPerThread>(sA[kk][pr][0], sA[kk][pr][1], sA[kk][pr][2], &sB[kk][cg],
                                   &sS[kk][cg], kLanes, acc);
    }
    const int j = pair0 + pr;
    if (j >= pairs) return;
#pragma unroll
    for (int t = 0; t < kPerThread; ++t) {
        const int col = col0 + cg + t * kLanes;
        if (col >= nc) continue;
        mg_3m_result(acc[0][t], acc[1][t], acc[2][t], G[(size_t)j * 2 * nc + col],
                     G[(size_t)j * 2 * nc + nc + col]);
    }
}

// A G term near the pole in FP64: G from its float-float value, wtilde and
// I_eps from the inputs.  Out of line, returning whole pairs.
static __device__ __noinline__ TermPair mg_pole_pair(const Problem &p, df2 d, float thr, int row0,
                                                     int ig, int iw, df2 Gr, df2 Gi, TermPair t) {
    const double wx = __ldg(p.wx + iw);
    for (int g = 0; g < 2; ++g) {
        if ((g == 0 ? d.h.x : d.h.y) >= thr) continue;
        const int row = min(row0 + g, p.ng - 1);
        const double2 wt = __ldg(p.wt + (size_t)row * p.nc + ig);
        const double2 ie = __ldg(p.ieps + (size_t)row * p.nc + ig);
        const double2 Gv = make_double2(to_double(df2_lane(Gr, g)), to_double(df2_lane(Gi, g)));
        const double2 A = cmul(Gv, cmul(wt, ie));
        const double wr = wx - wt.x;
        const double r = 1.0 / (wr * wr + wt.y * wt.y);
        df2_set_lane(t.re, g, split((A.x * wr - A.y * wt.y) * r));
        df2_set_lane(t.im, g, split((A.y * wr + A.x * wt.y) * r));
    }
    return t;
}

// The frequency pass: one block per row pair, threads over ig; the row
// tile's sum of G Q conj(wdiff) / |wdiff|^2 per frequency into its partial.
template <int NWC>
__global__ void __launch_bounds__(128) mg_freq_kernel(Problem p, Partials part, SplitPlanes s,
                                                      int wx_band, const float4 *__restrict__ G,
                                                      int row_tile0) {
    constexpr int THREADS = 128, K = NWC * 2;
    __shared__ double red[(THREADS / 32) * K];
    __shared__ double S[K];
    const int j = row_tile0 + blockIdx.x;
    const int iw0 = blockIdx.y * NWC;
    const int nc = p.nc, row0 = 2 * j;
    df wx[NWC];
    float thr[NWC];
#pragma unroll
    for (int w = 0; w < NWC; ++w) {
        const float2 x = s.wx[(size_t)wx_band * p.nw + min(iw0 + w, p.nw - 1)];
        wx[w] = {x.x, x.y};
        thr[w] = 1e-6f * x.x * x.x;
    }
    const df2 z = {f2(0.f, 0.f), f2(0.f, 0.f)};
    df2 acc[NWC][2];
#pragma unroll
    for (int w = 0; w < NWC; ++w) acc[w][0] = acc[w][1] = z;
    const float4 *rp = s.rows + (size_t)j * 4 * nc;
    const float4 *gp = G + (size_t)j * 2 * nc;
    for (int ig = threadIdx.x; ig < nc; ig += THREADS) {
        const float4 vr = __ldg(rp + ig), vi = __ldg(rp + nc + ig);
        const float4 vqr = __ldg(rp + 2 * nc + ig), vqi = __ldg(rp + 3 * nc + ig);
        const float4 g4r = __ldg(gp + ig), g4i = __ldg(gp + nc + ig);
        const df2 wtr = {f2(vr.x, vr.y), f2(vr.z, vr.w)}, wti = {f2(vi.x, vi.y), f2(vi.z, vi.w)};
        const df2 qr = {f2(vqr.x, vqr.y), f2(vqr.z, vqr.w)};
        const df2 qi = {f2(vqi.x, vqi.y), f2(vqi.z, vqi.w)};
        const df2 Gr = {f2(g4r.x, g4r.y), f2(g4r.z, g4r.w)};
        const df2 Gi = {f2(g4i.x, g4i.y), f2(g4i.z, g4i.w)};
        const df2 Ar = df2_sub(df2_mul(Gr, qr), df2_mul(Gi, qi));  // A = G Q
        const df2 Ai = df2_add(df2_mul(Gr, qi), df2_mul(Gi, qr));
        const df2 wti2 = df2_mul(wti, wti);
        const df2 Ai_wti = df2_mul(Ai, wti), Ar_wti = df2_mul(Ar, wti);
#pragma unroll
        for (int w = 0; w < NWC; ++w) {
            const df2 wr = df2_norm(df2_sub(df2_bcast(wx[w]), wtr));  // Re(wdiff)
            const df2 d = df2_add(df2_sqr(wr), wti2);                  // |wdiff|^2
            const df2 r = df2_rcp(d);
            TermPair t;
            t.re = df2_mul(df2_sub(df2_mul(Ar, wr), Ai_wti), r);
            t.im = df2_mul(df2_add(df2_mul(Ai, wr), Ar_wti), r);
            if (!(d.h.x >= thr[w]) || !(d.h.y >= thr[w]))
                t = mg_pole_pair(p, d, thr[w], row0, ig, min(iw0 + w, p.nw - 1), Gr, Gi, t);
            acc[w][0] = df2_add(acc[w][0], t.re);
            acc[w][1] = df2_add(acc[w][1], t.im);
        }
    }
    // Lanes are the pair's rows; a row past ngpown has G = 0 (c = 0).
    double v[K];
#pragma unroll
    for (int w = 0; w < NWC; ++w)
#pragma unroll
        for (int ri = 0; ri < 2; ++ri)
            v[w * 2 + ri] = to_double(df2_lane(acc[w][ri], 0)) + to_double(df2_lane(acc[w][ri], 1));
    block_reduce<K, THREADS>(v, red, S);
    const int w = threadIdx.x;
    if (w < NWC && iw0 + w < p.nw)
        part.ach[(long long)(iw0 + w) * part.ach_seg + part.ach_tile0 + j] =
            make_double2(S[w * 2], S[w * 2 + 1]);
}

// G's row-pair planes (re, im; lanes the pair's rows, hi then lo) from an
// FP64 G [ng][nc]; a row past ngpown is 0.
__global__ void __launch_bounds__(kThreads) mg_planes_kernel(const double2 *G, int ng, int nc,
                                                             float4 *Gp) {
    const int pairs = (ng + 1) / 2;
    const size_t n = (size_t)pairs * nc;
    for (size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (size_t)gridDim.x * kThreads) {
        const size_t j = i / nc, col = i % nc;
        const double2 g0 = G[2 * j * nc + col];
        const double2 g1 = 2 * j + 1 < (size_t)ng ? G[(2 * j + 1) * nc + col] : make_double2(0.0, 0.0);
        const df a0 = split_bits(g0.x), a1 = split_bits(g1.x);
        const df b0 = split_bits(g0.y), b1 = split_bits(g1.y);
        Gp[j * 2 * nc + col] = make_float4(a0.h, a1.h, a0.l, a1.l);
        Gp[j * 2 * nc + nc + col] = make_float4(b0.h, b1.h, b0.l, b1.l);
    }
}

// M_2[j][ig] = Q conj(wdiff) / |wdiff|^2 at iw = 2 for row pair j, in
// float-float lanes (FP64 from the inputs within 1e-3 |wx| of the pole),
// stored as two planes (re, im) per row pair.
static __device__ __noinline__ TermPair mg_pole_m2(const Problem &p, df2 d, float thr, int row0,
                                                   int ig, TermPair t) {
    const double wx = __ldg(p.wx + 2);
    for (int g = 0; g < 2; ++g) {
        if ((g == 0 ? d.h.x : d.h.y) >= thr) continue;
        const int row = min(row0 + g, p.ng - 1);
        const double2 wt = __ldg(p.wt + (size_t)row * p.nc + ig);
        const double2 Q = cmul(wt, __ldg(p.ieps + (size_t)row * p.nc + ig));
        const double wr = wx - wt.x;
        const double r = 1.0 / (wr * wr + wt.y * wt.y);
        df2_set_lane(t.re, g, split((Q.x * wr - Q.y * wt.y) * r));
        df2_set_lane(t.im, g, split((Q.y * wr + Q.x * wt.y) * r));
    }
    return t;
}

// M_2 of row pair j, column ig (both rows as the lanes).
__device__ __forceinline__ TermPair m2_pair(const Problem &p, const SplitPlanes &s, df wx,
                                            float thr, size_t j, size_t ig) {
    const size_t nc = (size_t)p.nc;
    const float4 *rp = s.rows + j * 4 * nc;
    const float4 vr = __ldg(rp + ig), vi = __ldg(rp + nc + ig);
    const float4 vqr = __ldg(rp + 2 * nc + ig), vqi = __ldg(rp + 3 * nc + ig);
    const df2 wtr = {f2(vr.x, vr.y), f2(vr.z, vr.w)}, wti = {f2(vi.x, vi.y), f2(vi.z, vi.w)};
    const df2 qr = {f2(vqr.x, vqr.y), f2(vqr.z, vqr.w)};
    const df2 qi = {f2(vqi.x, vqi.y), f2(vqi.z, vqi.w)};
    const df2 wr = df2_norm(df2_sub(df2_bcast(wx), wtr));
    const df2 d = df2_add(df2_sqr(wr), df2_mul(wti, wti));
    const df2 r = df2_rcp(d);
    TermPair t;
    t.re = df2_mul(df2_sub(df2_mul(qr, wr), df2_mul(qi, wti)), r);
    t.im = df2_mul(df2_add(df2_mul(qi, wr), df2_mul(qr, wti)), r);
    if (!(d.h.x >= thr) || !(d.h.y >= thr)) t = mg_pole_m2(p, d, thr, (int)(2 * j), (int)ig, t);
    return t;
}

__global__ void __launch_bounds__(kThreads) mg_m2_kernel(Problem p, SplitPlanes s, int wx_band,
                                                         float4 *M2) {
    const int pairs = (p.ng + 1) / 2;
    const size_t nc = (size_t)p.nc;
    const float2 x = s.wx[(size_t)wx_band * p.nw + 2];
    const df wx = {x.x, x.y};
    const float thr = 1e-6f * x.x * x.x;
    const size_t n = (size_t)pairs * nc;
    for (size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (size_t)gridDim.x * kThreads) {
        const size_t j = i / nc, ig = i % nc;
        const TermPair t = m2_pair(p, s, wx, thr, j, ig);
        M2[j * 2 * nc + ig] = make_float4(t.re.h.x, t.re.h.y, t.re.l.x, t.re.l.y);
        M2[j * 2 * nc + nc + ig] = make_float4(t.im.h.x, t.im.h.y, t.im.l.x, t.im.l.y);
    }
}

// The same M_2 as FP64 rows M[r][ig] (ng x nc), for the tensor-core
// per-band GEMM of the mixed path: the float-float lanes assembled into
// doubles on the integer pipes (no FP64 instruction but at the pole).
__global__ void __launch_bounds__(kThreads) mg_m2_fp64_kernel(Problem p, SplitPlanes s,
                                                              int wx_band, double2 *M) {
    const int pairs = (p.ng + 1) / 2;
    const size_t nc = (size_t)p.nc;
    const float2 x = s.wx[(size_t)wx_band * p.nw + 2];
    const df wx = {x.x, x.y};
    const float thr = 1e-6f * x.x * x.x;
    const size_t n = (size_t)pairs * nc;
    for (size_t i = (size_t)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (size_t)gridDim.x * kThreads) {
        const size_t j = i / nc, ig = i % nc;
        const TermPair t = m2_pair(p, s, wx, thr, j, ig);
        M[2 * j * nc + ig] = make_double2(oz_df_to_double(t.re.h.x, t.re.l.x),
                                          oz_df_to_double(t.im.h.x, t.im.l.x));
        if (2 * j + 1 < (size_t)p.ng)
            M[(2 * j + 1) * nc + ig] = make_double2(oz_df_to_double(t.re.h.y, t.re.l.y),
                                                    oz_df_to_double(t.im.h.y, t.im.l.y));
    }
}

constexpr int kHChunks = 16;   // column chunks of the H sum (summed in order afterwards)

// Hp[z][k][j] = sum over columns of chunk z of aqsn[k][ig] M_2[j][ig]:
// both rows of pair j as the lanes, the band value broadcast.  Grid: x row
// pair blocks, y band blocks, z column chunks.
__global__ void __launch_bounds__(kGemmThreads, kHMinBlocks) mg_gemm_h_kernel(
    int nbands, int pairs, int nc, int chunk, const float4 *__restrict__ M2,
    const float4 *__restrict__ band, float4 *__restrict__ Hp) {
    __shared__ float4 sA[kStep][kPairs][3];
    __shared__ float4 sB[kStep][kHBands];
    __shared__ float2 sS[kStep][kHBands];
    constexpr int kPerThread = kHBands / kLanes;
    const int tid = threadIdx.x;
    const int pr = tid / kLanes, cg = tid % kLanes;
    const int pair0 = blockIdx.x * kPairs, band0 = blockIdx.y * kHBands;
    const int ig_begin = blockIdx.z * chunk, ig_end = min(nc, ig_begin + chunk);
    const df2 z = {f2(0.f, 0.f), f2(0.f, 0.f)};
    df2 acc[3][kPerThread];
#pragma unroll
    for (int t = 0; t < kPerThread; ++t) acc[0][t] = acc[1][t] = acc[2][t] = z;
    const float4 zero4 = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int ig0 = ig_begin; ig0 < ig_end; ig0 += kStep) {
        const int kc = min(kStep, ig_end - ig0);
        __syncthreads();
        for (int i = tid; i < kStep * kPairs; i += kGemmThreads) {
            const int pp = i / kStep, kk = i % kStep;
            float4 re = zero4, im = zero4;
            if (kk < kc && pair0 + pp < pairs) {
                const float4 *m = M2 + (size_t)(pair0 + pp) * 2 * nc + ig0 + kk;
                re = m[0];
                im = m[nc];
            }
            mg_stage_a(re, im, sA[kk][pp]);
        }
        for (int i = tid; i < kStep * kHBands; i += kGemmThreads) {
            const int bb = i / kStep, kk = i % kStep;
            float4 v = zero4;
            if (kk < kc && band0 + bb < nbands) v = band[(size_t)(band0 + bb) * nc + ig0 + kk];
            mg_stage_b(v, &sB[kk][bb], &sS[kk][bb]);
        }
        __syncthreads();
        for (int kk = 0; kk < kc; ++kk)
            mg_3m_step<kPerThread>(sA[kk][pr][0], sA[kk][pr][1], sA[kk][pr][2], &sB[kk][cg],
                                   &sS[kk][cg], kLanes, acc);
    }
    const int j = pair0 + pr;
    if (j >= pairs) return;
#pragma unroll
    for (int t = 0; t < kPerThread; ++t) {
        const int k = band0 + cg + t * kLanes;
        if (k >= nbands) continue;
        float4 *o = Hp + (((size_t)blockIdx.z * nbands + k) * pairs + j) * 2;
        mg_3m_result(acc[0][t], acc[1][t], acc[2][t], o[0], o[1]);
    }
}

// acht_n1_loc partials: band b0 + k, row tile j: sum_rows c H with H the
// chunk sums of Hp added in chunk order.
__global__ void __launch_bounds__(kThreads) mg_n1_kernel(Partials part, int b0, int K, int pairs,
                                                         int chunks, const float4 *cpl,
                                                         const float4 *Hp) {
    const long long n = (long long)K * pairs;
    const df2 z = {f2(0.f, 0.f), f2(0.f, 0.f)};
    for (long long i = (long long)blockIdx.x * kThreads + threadIdx.x; i < n;
         i += (long long)gridDim.x * kThreads) {
        const int k = (int)(i / pairs), j = (int)(i % pairs);
        df2 hr = z, hi = z;
        for (int c = 0; c < chunks; ++c) {
            const float4 *h = Hp + (((size_t)c * K + k) * pairs + j) * 2;
            const float4 a = h[0], b = h[1];
            hr = df2_add(hr, df2{f2(a.x, a.y), f2(a.z, a.w)});
            hi = df2_add(hi, df2{f2(b.x, b.y), f2(b.z, b.w)});
        }
        const float4 a = cpl[i * 2], b = cpl[i * 2 + 1];
        const df2 cr = {f2(a.x, a.y), f2(a.z, a.w)}, ci = {f2(b.x, b.y), f2(b.z, b.w)};
        const df2 pr = df2_sub(df2_mul(cr, hr), df2_mul(ci, hi));
        const df2 pi = df2_add(df2_mul(cr, hi), df2_mul(ci, hr));
        part.n1[(long long)(b0 + k) * part.n1_seg + j] =
            make_double2(to_double(df2_lane(pr, 0)) + to_double(df2_lane(pr, 1)),
                         to_double(df2_lane(pi, 0)) + to_double(df2_lane(pi, 1)));
    }
}

int grid_for(long long n) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (n + kThreads - 1) / kThreads;
    const long long cap = (long long)(sms > 0 ? sms : 132) * 8;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

template <int NWC>
cudaError_t launch_freq_t(const Problem &p, const Partials &part, const SplitPlanes &s, int wx_band,
                          const float4 *G, RowTiles r, cudaStream_t st) {
    dim3 grid((unsigned)(r.end - r.begin), (unsigned)ceil_div(p.nw, NWC));
    mg_freq_kernel<NWC><<<grid, 128, 0, st>>>(p, part, s, wx_band, G, r.begin);
    count_launch();
    return cudaGetLastError();
}

float4 *planes_c(void *ws) { return static_cast<float4 *>(ws); }
float4 *planes_g(const Problem &p, void *ws, int K) {
    return reinterpret_cast<float4 *>(static_cast<char *>(ws) +
                                      align_up(sizeof(float4) * 2 * (size_t)K * row_pairs(p)));
}

}  // namespace

size_t mixed_gemm_bytes(const Problem &p, int bands, bool want_n1) {
    size_t b = align_up(sizeof(float4) * 2 * (size_t)bands * row_pairs(p)) +
               align_up(sizeof(float4) * 2 * (size_t)row_pairs(p) * p.nc);
    if (want_n1)
        b += align_up(sizeof(float4) * 2 * (size_t)row_pairs(p) * p.nc) +
             align_up(sizeof(float4) * 2 * (size_t)kHChunks * bands * row_pairs(p));
    return b;
}

gpp_status mixed_gemm_band_sum(const Problem &p, const Partials &part, void *split_ws, void *ws,
                               int b0, int b1, cudaStream_t st) {
    const SplitPlanes s = split_planes_at(p, split_ws);
    const int K = b1 - b0, pairs = row_pairs(p);
    if (K <= 0 || pairs <= 0) return GPP_OK;
    float4 *cpl = planes_c(ws);
    mg_coeff_kernel<<<grid_for((long long)K * pairs), kThreads, 0, st>>>(p, b0, K, cpl, part.err);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mg_coeff_kernel");
    if (ceil_div(p.nc, kCols) > 65535)
        return set_error(GPP_ERR_UNSUPPORTED, "ncouls too large for the band-sum GEMM grid");
    dim3 grid((unsigned)ceil_div(pairs, kPairs), (unsigned)ceil_div(p.nc, kCols));
    mg_gemm_kernel<<<grid, kGemmThreads, 0, st>>>(K, pairs, p.nc, cpl, s.band + (size_t)b0 * p.nc,
                                              planes_g(p, ws, K));
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mg_gemm_kernel");
    return GPP_OK;
}

gpp_status mixed_gemm_planes_from(const Problem &p, void *ws, int b0, int b1, const double2 *G,
                                  cudaStream_t st) {
    const int K = b1 - b0, pairs = row_pairs(p);
    if (K <= 0 || pairs <= 0) return GPP_OK;
    mg_planes_kernel<<<grid_for((long long)pairs * p.nc), kThreads, 0, st>>>(G, p.ng, p.nc,
                                                                          planes_g(p, ws, K));
    count_launch();
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? GPP_OK : cuda_fail(e, "mg_planes_kernel");
}

gpp_status mixed_gemm_rows(const Problem &p, const Partials &part, void *split_ws, void *ws, int b0,
                           int b1, cudaStream_t st, RowTiles rows) {
    const SplitPlanes s = split_planes_at(p, split_ws);
    const RowTiles rt = rows.clip(row_pairs(p));
    if (rt.end <= rt.begin || b1 <= b0) return GPP_OK;
    const float4 *G = planes_g(p, ws, b1 - b0);
    const int nwc = p.nw <= 4 ? p.nw : 8;
    cudaError_t e;
    switch (nwc) {
        case 1: e = launch_freq_t<1>(p, part, s, b0, G, rt, st); break;
        case 2: e = launch_freq_t<2>(p, part, s, b0, G, rt, st); break;
        case 3: e = launch_freq_t<3>(p, part, s, b0, G, rt, st); break;
        case 4: e = launch_freq_t<4>(p, part, s, b0, G, rt, st); break;
        default: e = launch_freq_t<8>(p, part, s, b0, G, rt, st); break;
    }
    if (e != cudaSuccess) return cuda_fail(e, "mg_freq_kernel");
    return GPP_OK;
}

gpp_status mixed_m2_fp64(const Problem &p, void *split_ws, int wx_band, double2 *M,
                         cudaStream_t st) {
    const int pairs = row_pairs(p);
    if (pairs <= 0) return GPP_OK;
    const SplitPlanes s = split_planes_at(p, split_ws);
    mg_m2_fp64_kernel<<<grid_for((long long)pairs * p.nc), kThreads, 0, st>>>(p, s, wx_band, M);
    count_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mg_m2_fp64_kernel");
    return GPP_OK;
}

gpp_status mixed_gemm_per_band(const Problem &p, const Partials &part, void *split_ws, void *ws,
                               int b0, int b1, cudaStream_t st) {
    const int K = b1 - b0, pairs = row_pairs(p);
    if (K <= 0 || pairs <= 0 || !part.n1) return GPP_OK;
    const SplitPlanes s = split_planes_at(p, split_ws);
    const size_t plane = align_up(sizeof(float4) * 2 * (size_t)pairs * p.nc);
    float4 *M2 = reinterpret_cast<float4 *>(reinterpret_cast<char *>(planes_g(p, ws, K)) + plane);
    float4 *Hp = reinterpret_cast<float4 *>(reinterpret_cast<char *>(M2) + plane);
    mg_m2_kernel<<<grid_for((long long)pairs * p.nc), kThreads, 0, st>>>(p, s, b0, M2);
    count_launch();
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mg_m2_kernel");
    const int chunk = ceil_div(ceil_div(p.nc, kHChunks), kStep) * kStep;
    const int chunks = ceil_div(p.nc, chunk);
    if (ceil_div(K, kHBands) > 65535)
        return set_error(GPP_ERR_UNSUPPORTED, "too many bands for the per-band product grid");
    dim3 grid((unsigned)ceil_div(pairs, kPairs), (unsigned)ceil_div(K, kHBands), (unsigned)chunks);
    mg_gemm_h_kernel<<<grid, kGemmThreads, 0, st>>>(K, pairs, p.nc, chunk, M2,
                                                s.band + (size_t)b0 * p.nc, Hp);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mg_gemm_h_kernel");
    mg_n1_kernel<<<grid_for((long long)K * pairs), kThreads, 0, st>>>(part, b0, K, pairs, chunks,
                                                                      planes_c(ws), Hp);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "mg_n1_kernel");
    return GPP_OK;
}

}  // namespace gpp
