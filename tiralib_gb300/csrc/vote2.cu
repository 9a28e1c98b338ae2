// 2D tensor voting (TK and ATV) on sm_103a and its C ABI.
//
// Reference path replaced (tira/functions/tensorvote.h):
//   tira::cuda::tensorvote :2201 -> evals2_symmetric / evecs2polar_symmetric
//   (eigen.h:769,828, each with host round trips) -> tensorvote_tk :2126
//   (cpu::build_neighbors2d :1223 on the host, upload, global_tensorvote_tk
//   :2072 with threadIdx.x on the SLOW axis, so every load is strided, and a
//   cos/sin of the voter angle per pair) or tensorvote_atv :2029.
//
// Here: one prep kernel solves every pixel's 2x2 once (eigen.h semantics) and
// stores the voter record (cos th1, sin th1, stick scale, lambda0); the vote
// kernel maps x (fast axis) to threadIdx.x so voter loads coalesce, and
// streams the Neighbor2D table through shared memory so each entry is a
// broadcast read.  The table itself is built on the host with the
// reference's float arithmetic (it is O(w^2 samples) and tiny).
#include "tvgb_internal.cuh"
#include "eig_device.cuh"
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <vector>

namespace tvgb {

struct Nb2 {             // tira::Neighbor2D, 48 bytes (tensorvote.h:776)
    int du, dv;
    float dx, dy, c1, c2, Ra, Rb, Rc, Va, Vb, Vc;
};
static_assert(sizeof(Nb2) == 48, "Neighbor2D must be 48 bytes");

// ---------------------------------------------------------------- host table (float steps of the reference)
static float atten_h(float dist, float sigma) {            // atv_attenuation, :35
    if (sigma == 0.0f) return (double(dist) > 1e-12) ? 0.0f : 1.0f;
    return std::exp(-(dist * dist) / (sigma * sigma));
}
static float stick_norm_2d_h(float s1, float s2, unsigned p) {   // tk_stick_norm_2d, :843
    if (p < 1) p = 1;
    float r = 1.0f;
    for (unsigned k = 1; k <= p; ++k) r *= float(2 * k) / float(2 * k - 1);
    return r / (float(3.14159265358979323846) * (s1 * s1 + s2 * s2));
}
static void stickvote_2d_h(float rx, float ry, float s1, float s2, unsigned power, float theta, float& Va, float& Vb,
                           float& Vc) {                     // tk_stickvote_2d, :872
    const float qx = std::cos(theta), qy = std::sin(theta);
    const float dist = std::sqrt(rx * rx + ry * ry);
    float dx = 0.0f, dy = 0.0f;
    if (dist != 0.0f) { dx = rx / dist; dy = ry / dist; }
    const float qTd = qx * dx + qy * dy;
    unsigned p = power < 1 ? 1 : power;
    const float c1 = atten_h(dist, s1), c2 = atten_h(dist, s2);
    const float q2 = qTd * qTd, t1 = 1.0f - q2, t2 = q2;
    float D;
    if (p == 1) D = c1 * t1 + c2 * t2;
    else { float e1 = t1, e2 = t2; for (unsigned i = 1; i < p; ++i) { e1 *= t1; e2 *= t2; } D = c1 * e1 + c2 * e2; }
    const float factor = D * stick_norm_2d_h(s1, s2, power);
    const float Ra = 1 - 2 * dx * dx, Rb = -2 * dx * dy, Rc = 1 - 2 * dy * dy;
    const float Rqx = Ra * qx + Rb * qy, Rqy = Rb * qx + Rc * qy;
    Va = Rqx * Rqx * factor; Vb = Rqx * Rqy * factor; Vc = Rqy * Rqy * factor;
}

static int build_table(int w, float s1, float s2, unsigned power, unsigned samples, bool stick, bool plate, Nb2* out) {
    if (w <= 0) return 0;
    const int hw = w / 2;
    const float inv1 = s1 > 0 ? 1.0f / (s1 * s1) : 0.0f, inv2 = s2 > 0 ? 1.0f / (s2 * s2) : 0.0f;
    int k = 0;
    for (int dv = -hw; dv <= hw; dv++)
        for (int du = -hw; du <= hw; du++) {
            Nb2 e{};
            e.du = du; e.dv = dv;
            const float l2 = float(du * du + dv * dv);
            if (stick) {
                if (l2 != 0.0f) { const float il = 1.0f / std::sqrt(l2); e.dx = float(du) * il; e.dy = float(dv) * il; }
                e.c1 = s1 == 0.0f ? (l2 > 1e-12f ? 0.0f : 1.0f) : std::exp(-l2 * inv1);
                e.c2 = s2 == 0.0f ? (l2 > 1e-12f ? 0.0f : 1.0f) : std::exp(-l2 * inv2);
                e.Ra = 1.0f - 2.0f * e.dx * e.dx; e.Rb = 0.0f - 2.0f * e.dx * e.dy; e.Rc = 1.0f - 2.0f * e.dy * e.dy;
            }
            if (plate && samples > 0) {      // tk_plate_numerical (2D), :1048
                const float dth = float(3.14159265358979323846 / double(float(samples)));
                float a = 0, b = 0, c = 0;
                for (unsigned i = 0; i < samples; ++i) {
                    float va, vb, vc;
                    stickvote_2d_h(float(du), float(dv), s1, s2, power, dth * float(i), va, vb, vc);
                    a += va; b += vb; c += vc;
                }
                const float wb = float(3.14159265358979323846) / float(samples);
                e.Va = a * wb; e.Vb = b * wb; e.Vc = c * wb;
            }
            if (out) out[k] = e;
            k++;
        }
    return k;
}

// ---------------------------------------------------------------- kernels
// voter record: (cos th1, sin th1, stick scale, lambda0); ATV adds (l1, cos th0, sin th0)
__global__ void k_prep2(const float4* __restrict__ in, size_t n, float4* __restrict__ V, float4* __restrict__ W) {
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
        const float4 m = __ldg(in + i);
        float l0, l1, t0, t1;
        eval2_d(m.x, m.y, m.w, l0, l1);
        evec2polar_d(m.x, m.y, m.w, l0, t0, t1);
        float scale = fabsf(l1) - fabsf(l0);
        if (l1 < 0.0f) scale = -scale;                     // tk_stick_window, :996-997
        V[i] = make_float4(cosf(t1), sinf(t1), scale, l0);
        if (W) W[i] = make_float4(l1, cosf(t0), sinf(t0), 0.0f);
    }
}

constexpr int V2X = 32, V2Y = 8, NB_CHUNK = 512;

template <bool STICK, bool PLATE>
__global__ void __launch_bounds__(V2X * V2Y) k_vote2_tk(const float4* __restrict__ V, const Nb2* __restrict__ nb, int nbc,
                                                         int s0, int s1, float eta_s, unsigned power, float4* __restrict__ out) {
    __shared__ Nb2 snb[NB_CHUNK];
    const int x = blockIdx.x * V2X + threadIdx.x;    // fast axis (x1)
    const int y = blockIdx.y * V2Y + threadIdx.y;    // slow axis (x0)
    const int tid = threadIdx.y * V2X + threadIdx.x;
    float sa = 0, sb = 0, sc = 0, pa = 0, pb = 0, pc = 0;
    for (int c0 = 0; c0 < nbc; c0 += NB_CHUNK) {
        const int cn = min(NB_CHUNK, nbc - c0);
        __syncthreads();
        for (int i = tid; i < cn; i += V2X * V2Y) snb[i] = nb[c0 + i];
        __syncthreads();
        for (int k = 0; k < cn; ++k) {
            const Nb2& e = snb[k];
            const int r0 = y + e.dv, r1 = x + e.du;
            if ((unsigned)r0 >= (unsigned)s0 || (unsigned)r1 >= (unsigned)s1) continue;
            const float4 v = __ldg(V + size_t(r0) * s1 + r1);
            if (STICK) {
                const float qTd = v.x * e.dx + v.y * e.dy;
                const float q2 = qTd * qTd, t1 = 1.0f - q2, t2 = q2;
                float D;
                if (power == 1) D = e.c1 * t1 + e.c2 * t2;
                else { float e1 = t1, e2 = t2; for (unsigned i = 1; i < power; ++i) { e1 *= t1; e2 *= t2; } D = e.c1 * e1 + e.c2 * e2; }
                const float Rqx = e.Ra * v.x + e.Rb * v.y, Rqy = e.Rb * v.x + e.Rc * v.y;
                const float f = D * eta_s * v.z;
                sa = fmaf(f * Rqx, Rqx, sa); sb = fmaf(f * Rqx, Rqy, sb); sc = fmaf(f * Rqy, Rqy, sc);
            }
            if (PLATE && v.w != 0.0f) {
                pa = fmaf(v.w, e.Va, pa); pb = fmaf(v.w, e.Vb, pb); pc = fmaf(v.w, e.Vc, pc);
            }
        }
    }
    if (x < s1 && y < s0) out[size_t(y) * s1 + x] = make_float4(sa + pa, sb + pb, sb + pb, sc + pc);
}

// Staged variant for windows whose voter tile fits in shared memory: a CTA
// of 32 x TY threads owns 32 x (TY V2R) receivers (V2R rows per thread, TY
// apart) and reads their voters from a (32 + 2 h) x (TY V2R + 2 h) tile
// staged once, zero outside the image, so the table loop has no bounds checks
// and each table entry (a warp-uniform broadcast) serves V2R receivers.  h
// bounds |du|, |dv| over the table.  The table streams through shared memory
// in chunks of NBC entries.  Measured at 512^2 (C1, 20-step bench): TY = 8
// (256 CTAs, 0.56 of a wave) 0.083 ms, TY = 4 0.092 ms, TY = 2 (1024 CTAs,
// all resident) 0.094 ms: the kernel runs at the pace its warps' dependent
// chains allow, and smaller CTAs buy no more warps per SM.
//
// Per pair, FP32 operations (the pipe that bounds the kernel): the stick
// weight D = c1 (1 - q^2)^p + c2 (q^2)^p is, for p = 1, c1 + (c2 - c1) q^2
// (one FMA with c2 - c1 formed once per entry); the reflected orientation
// R q = q - 2 (q.d) d costs a multiply and two FMAs instead of the four
// operations of the entry's (Ra, Rb, Rc) matrix product.  16 operations per
// pair with the plate, against 19 for the reference's literal expressions;
// both agree to FP32 rounding (0.092 -> 0.083 ms at C1).  A packed form
// (two receiver rows per FFMA2 from a paired-row tile, pre-broadcast table
// entries) measured 0.092 ms: a packed instruction holds the FP32 pipe as
// long as two scalar ones, and its larger tile and entry loads cost more than
// the issue slots it saves.
template <int V2R, int TY, int NBC, bool STICK, bool PLATE, bool P1>
__global__ void __launch_bounds__(V2X * TY) k_vote2_tks(const float4* __restrict__ V, const Nb2* __restrict__ nb,
                                                        int nbc, int s0, int s1, int h, float eta_s, unsigned power,
                                                        float4* __restrict__ out) {
    extern __shared__ __align__(16) float4 sm2[];
    Nb2* snb = reinterpret_cast<Nb2*>(sm2);                       // NBC entries
    float4* tile = sm2 + NBC * sizeof(Nb2) / sizeof(float4);      // TW x TH voters
    constexpr int NT = V2X * TY;
    const int TW = V2X + 2 * h, TH = TY * V2R + 2 * h;
    const int x0 = blockIdx.x * V2X, y0 = blockIdx.y * (TY * V2R);
    const int tid = threadIdx.y * V2X + threadIdx.x;
    for (int e = tid; e < TW * TH; e += NT) {
        const int r = e / TW, c = e - r * TW;
        const int gy = y0 - h + r, gx = x0 - h + c;
        tile[e] = ((unsigned)gy < (unsigned)s0 && (unsigned)gx < (unsigned)s1) ? __ldg(V + size_t(gy) * s1 + gx)
                                                                               : make_float4(0.f, 0.f, 0.f, 0.f);
    }
    float sa[V2R], sb[V2R], sc[V2R], pa[V2R], pb[V2R], pc[V2R];
#pragma unroll
    for (int j = 0; j < V2R; ++j) { sa[j] = sb[j] = sc[j] = pa[j] = pb[j] = pc[j] = 0.0f; }
    // receiver j of this thread: (x0 + tx, y0 + ty + TY j); its voter at (du, dv) is tile[ty + TY j + h + dv][tx + h + du]
    const float4* base = tile + (threadIdx.y + h) * TW + threadIdx.x + h;
    for (int c0 = 0; c0 < nbc; c0 += NBC) {
        const int cn = min(NBC, nbc - c0);
        __syncthreads();
        for (int i = tid; i < cn; i += NT) snb[i] = nb[c0 + i];
        __syncthreads();
#pragma unroll 2
        for (int k = 0; k < cn; ++k) {
            const Nb2& e = snb[k];
            const float4* vp = base + e.dv * TW + e.du;
            const float dc = e.c2 - e.c1;
#pragma unroll
            for (int j = 0; j < V2R; ++j) {
                const float4 v = vp[j * TY * TW];
                if (STICK) {
                    const float qTd = fmaf(v.x, e.dx, v.y * e.dy);
                    const float q2 = qTd * qTd;
                    float D;
                    if (P1) D = fmaf(dc, q2, e.c1);
                    else {
                        const float t1 = 1.0f - q2, t2 = q2;
                        float e1 = t1, e2 = t2;
                        for (unsigned i = 1; i < power; ++i) { e1 *= t1; e2 *= t2; }
                        D = e.c1 * e1 + e.c2 * e2;
                    }
                    const float k2 = -2.0f * qTd;
                    const float Rqx = fmaf(k2, e.dx, v.x), Rqy = fmaf(k2, e.dy, v.y);
                    const float f = D * v.z;
                    const float fx = f * Rqx;
                    sa[j] = fmaf(fx, Rqx, sa[j]); sb[j] = fmaf(fx, Rqy, sb[j]); sc[j] = fmaf(f * Rqy, Rqy, sc[j]);
                }
                if (PLATE) {   // v.w = 0 outside the image and for zero plates
                    pa[j] = fmaf(v.w, e.Va, pa[j]); pb[j] = fmaf(v.w, e.Vb, pb[j]); pc[j] = fmaf(v.w, e.Vc, pc[j]);
                }
            }
        }
    }
    const int x = x0 + threadIdx.x;
    if (x >= s1) return;
#pragma unroll
    for (int j = 0; j < V2R; ++j) {
        const int y = y0 + threadIdx.y + TY * j;
        if (y >= s0) break;
        const float a = fmaf(eta_s, sa[j], pa[j]), b = fmaf(eta_s, sb[j], pb[j]), c = fmaf(eta_s, sc[j], pc[j]);
        out[size_t(y) * s1 + x] = make_float4(a, b, b, c);
    }
}

// atv (2D, tensorvote.h:225) with atv_H (:161); out [a, b, c]
__device__ __forceinline__ void atv2_pair(float l0, float l1, float e0x, float e0y, float e1x, float e1y, float rx,
                                          float ry, float sigma, float& Va, float& Vb, float& Vc) {
    const float dist = sqrtf(rx * rx + ry * ry);
    const float c = sigma == 0.0f ? (dist > 1e-12f ? 0.0f : 1.0f) : expf(-(dist * dist) / (sigma * sigma));
    float dx = 0.0f, dy = 0.0f;
    if (dist != 0.0f) { dx = rx / dist; dy = ry / dist; }
    const float Ra = 1 - 2 * dx * dx, Rb = -2 * dx * dy, Rc = 1 - 2 * dy * dy;
    const float T1a = e1x * e1x, T1b = e1x * e1y, T1c = e1y * e1y;
    const float T0a = e0x * e0x + T1a, T0b = e0x * e0y + T1b, T0c = e0y * e0y + T1c;
    const float v0 = dx * (dx * T0a + dy * T0b) + dy * (dx * T0b + dy * T0c);
    const float v1 = dx * (dx * T1a + dy * T1b) + dy * (dx * T1b + dy * T1c);
    const float t0x = T0a * dx + T0b * dy, t0y = T0b * dx + T0c * dy;
    const float t1x = T1a * dx + T1b * dy, t1y = T1b * dx + T1c * dy;
    const float s1 = l1 - l0, i3 = 1.0f / 3.0f, i4 = 1.0f / 4.0f;
    float Ha = s1 * (T1a - i3 * (T1a * v1 + 2 * (t1x * t1x)));
    float Hb = s1 * (T1b - i3 * (T1b * v1 + 2 * (t1x * t1y)));
    float Hc = s1 * (T1c - i3 * (T1c * v1 + 2 * (t1y * t1y)));
    Ha += l0 * (T0a - i4 * (T0a * v0 + 2 * (t0x * t0x)));
    Hb += l0 * (T0b - i4 * (T0b * v0 + 2 * (t0x * t0y)));
    Hc += l0 * (T0c - i4 * (T0c * v0 + 2 * (t0y * t0y)));
    const float Ra2 = Ra * Ra, Rb2 = Rb * Rb, Rc2 = Rc * Rc, Rab = Ra * Rb, Rbc = Rb * Rc, Rac = Ra * Rc;
    Va = c * (Ra2 * Ha + 2 * Rab * Hb + Rb2 * Hc);
    Vb = c * (Rb2 * Hb + Rab * Ha + Rac * Hb + Rbc * Hc);
    Vc = c * (Rb2 * Ha + 2 * Rbc * Hb + Rc2 * Hc);
}

__global__ void __launch_bounds__(V2X * V2Y) k_vote2_atv(const float4* __restrict__ V, const float4* __restrict__ W,
                                                          int s0, int s1, int hw, float sigma, float4* __restrict__ out) {
    const int x = blockIdx.x * V2X + threadIdx.x, y = blockIdx.y * V2Y + threadIdx.y;
    if (x >= s1 || y >= s0) return;
    float oa = 0, ob = 0, oc = 0;
    for (int v = -hw; v <= hw; ++v) {
        const int r0 = y + v;
        if (r0 < 0 || r0 >= s0) continue;
        for (int u = -hw; u <= hw; ++u) {
            const int r1 = x + u;
            if (r1 < 0 || r1 >= s1) continue;
            const size_t i = size_t(r0) * s1 + r1;
            const float4 a = __ldg(V + i), b = __ldg(W + i);
            float va, vb, vc;
            atv2_pair(a.w, b.x, b.y, b.z, a.x, a.y, float(u), float(v), sigma, va, vb, vc);
            oa += va; ob += vb; oc += vc;
        }
    }
    out[size_t(y) * s1 + x] = make_float4(oa, ob, ob, oc);
}

// Tables the library builds itself stay on the device, one per (device,
// window, sigmas, power, samples, terms), so a repeated vote neither copies
// nor waits for its table.  At most kTableCache tables are kept (a parameter
// sweep beyond that builds and uploads the extra ones per call).
struct TableEntry {
    int dev, w, power, samples, stick, plate, nbc, h;
    float s1, s2;
    Nb2* table;
};
constexpr int kTableCache = 128;
static std::mutex g_tab_mu;
static std::vector<TableEntry> g_tabs;

static int cached_table(int w, float s1, float s2, unsigned power, unsigned samples, bool stick, bool plate,
                        const TableEntry*& hit) {
    hit = nullptr;
    int dev = 0;
    TVGB_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> g(g_tab_mu);
    for (const TableEntry& e : g_tabs)
        if (e.dev == dev && e.w == w && e.s1 == s1 && e.s2 == s2 && e.power == int(power) &&
            e.samples == int(samples) && e.stick == int(stick) && e.plate == int(plate)) {
            hit = &e;
            return TVGB_OK;
        }
    if (int(g_tabs.size()) >= kTableCache) return TVGB_OK;
    std::vector<Nb2> t(size_t(w) * w);
    const int nbc = build_table(w, s1, s2, power, samples, stick, plate, t.data());
    int h = 0;
    for (int i = 0; i < nbc; ++i) h = std::max(h, std::max(std::abs(t[i].du), std::abs(t[i].dv)));
    Nb2* d = nullptr;
    if (nbc > 0) {
        TVGB_CUDA(cudaMalloc(&d, size_t(nbc) * sizeof(Nb2)));
        const cudaError_t e = cudaMemcpy(d, t.data(), size_t(nbc) * sizeof(Nb2), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(d);
            set_error("table upload failed: %s", cudaGetErrorString(e));
            return TVGB_ERR_CUDA;
        }
    }
    g_tabs.reserve(kTableCache);   // entries never move: hit stays valid
    g_tabs.push_back(TableEntry{dev, w, int(power), int(samples), int(stick), int(plate), nbc, h, s1, s2, d});
    hit = &g_tabs.back();
    return TVGB_OK;
}

// One TK vote of prepared voter records V (k_prep2) into out: the
// Neighbor2D table is the caller's (host or device) or the library's own
// (cached on the device); the staged kernel runs whenever the table's extent
// is known and its voter tile fits in shared memory.
static int vote2_tk_launch(const float4* V, const Nb2* host_or_dev_nb, int nbc, float s1, float s2, int power,
                           unsigned w, unsigned S0, unsigned S1, bool stick, bool plate, unsigned samples, float4* out,
                           cudaStream_t st) {
    const bool use_plate = plate && samples > 0;
    std::vector<Nb2> table;
    const Nb2* nbp = host_or_dev_nb;
    const TableEntry* cached = nullptr;
    if (!nbp) {
        TVGB_TRY(cached_table(int(w), s1, s2, unsigned(power), samples, stick, use_plate, cached));
        if (cached) {
            nbp = cached->table;
            nbc = cached->nbc;
        } else {
            table.resize(size_t(w) * w);
            nbc = build_table(int(w), s1, s2, unsigned(power), samples, stick, use_plate, table.data());
            nbp = table.data();
        }
    }
    DevArray dnb;
    TVGB_TRY(dnb.in(nbp, size_t(nbc) * sizeof(Nb2), st));
    const unsigned p = power < 1 ? 1u : unsigned(power);
    const float eta_s = stick_norm_2d_h(s1, s2, p);
    int h = -1;
    if (cached) {
        h = cached->h;
    } else if (!is_device_ptr(nbp)) {
        h = 0;
        for (int i = 0; i < nbc; ++i) h = std::max(h, std::max(std::abs(nbp[i].du), std::abs(nbp[i].dv)));
    }
    // staged kernel: 4 receivers per thread (each table entry serves 4), 32 x 8 threads per CTA
    constexpr int V2R = 4, TY = 8, V2NBC = 128;
    const size_t hh = size_t(h < 0 ? 0 : h);
    const size_t smem_s = V2NBC * sizeof(Nb2) + (V2X + 2 * hh) * (size_t(TY) * V2R + 2 * hh) * sizeof(float4);
    dim3 grid(ceil_div(S1, V2X), ceil_div(S0, V2Y)), blk(V2X, V2Y);
    {
        KernelTimer kt_("k_vote2_tk", st);
        if (h >= 0 && smem_s <= 200 * 1024) {
            const void* fn = nullptr;
            if (stick && use_plate) fn = p == 1 ? (const void*)k_vote2_tks<V2R, TY, V2NBC, true, true, true>
                                                : (const void*)k_vote2_tks<V2R, TY, V2NBC, true, true, false>;
            else if (stick) fn = p == 1 ? (const void*)k_vote2_tks<V2R, TY, V2NBC, true, false, true>
                                        : (const void*)k_vote2_tks<V2R, TY, V2NBC, true, false, false>;
            else fn = (const void*)k_vote2_tks<V2R, TY, V2NBC, false, true, true>;
            TVGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem_s)));
            dim3 gs(ceil_div(S1, V2X), ceil_div(S0, unsigned(TY * V2R))), bs(V2X, TY);
            const float4* vp = V;
            const Nb2* tp = dnb.get<Nb2>();
            int nbc_ = nbc, s0_ = int(S0), s1_ = int(S1), h_ = h;
            float eta_ = eta_s;
            unsigned p_ = p;
            float4* op = out;
            void* args[] = {&vp, &tp, &nbc_, &s0_, &s1_, &h_, &eta_, &p_, &op};
            TVGB_CUDA(cudaLaunchKernel(fn, gs, bs, args, smem_s, st));
        } else if (stick && use_plate) {
            k_vote2_tk<true, true><<<grid, blk, 0, st>>>(V, dnb.get<Nb2>(), nbc, int(S0), int(S1), eta_s, p, out);
        } else if (stick) {
            k_vote2_tk<true, false><<<grid, blk, 0, st>>>(V, dnb.get<Nb2>(), nbc, int(S0), int(S1), eta_s, p, out);
        } else {
            k_vote2_tk<false, true><<<grid, blk, 0, st>>>(V, dnb.get<Nb2>(), nbc, int(S0), int(S1), eta_s, p, out);
        }
        kt_.stop();
    }
    TVGB_LAUNCHED();
    if (!host_or_dev_nb && !cached) TVGB_CUDA(cudaStreamSynchronize(st));   // the host table must outlive its copy
    return TVGB_OK;
}

static int vote2_impl(float* t_out, const float* t_in, const Nb2* host_or_dev_nb, int nbc, float s1, float s2,
                      int power, unsigned w, unsigned S0, unsigned S1, bool stick, bool plate, unsigned samples,
                      bool is_atv, cudaStream_t st) {
    const size_t n = size_t(S0) * S1;
    DevArray din, dout;
    TVGB_TRY(din.in(t_in, n * 16, st));
    TVGB_TRY(dout.out(t_out, n * 16, st));
    TVGB_CHECK_ARG(reinterpret_cast<uintptr_t>(din.dev) % 16 == 0 && reinterpret_cast<uintptr_t>(dout.dev) % 16 == 0,
                   "2D tensor fields must be 16-byte aligned");
    if (!is_atv && !stick && !plate) {      // global_tensorvote_tk writes zeros (:2079-2085)
        TVGB_CUDA(cudaMemsetAsync(dout.dev, 0, n * 16, st));
        TVGB_TRY(dout.finish());
        return sync_if(din.owned || dout.owned, st);
    }
    Scratch sv, sw;
    TVGB_TRY(sv.alloc(n * 16, st));
    if (is_atv) TVGB_TRY(sw.alloc(n * 16, st));
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    size_t blocks = (n + 255) / 256;
    if (blocks > size_t(sms) * 16) blocks = size_t(sms) * 16;
    {
        KernelTimer kt_("k_prep2", st);
        k_prep2<<<unsigned(blocks ? blocks : 1), 256, 0, st>>>(din.get<float4>(), n, sv.get<float4>(),
                                                              is_atv ? sw.get<float4>() : nullptr);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    dim3 grid(ceil_div(S1, V2X), ceil_div(S0, V2Y)), blk(V2X, V2Y);
    if (is_atv) {
        {
            KernelTimer kt_("k_vote2_atv", st);
            k_vote2_atv<<<grid, blk, 0, st>>>(sv.get<float4>(), sw.get<float4>(), int(S0), int(S1), int(w / 2), s1,
                                              dout.get<float4>());
            kt_.stop();
        }
        TVGB_LAUNCHED();
    } else {
        TVGB_TRY(vote2_tk_launch(sv.get<float4>(), host_or_dev_nb, nbc, s1, s2, power, w, S0, S1, stick, plate, samples,
                                 dout.get<float4>(), st));
    }
    TVGB_TRY(dout.finish());
    return sync_if(din.owned || dout.owned, st);
}

}  // namespace tvgb

using namespace tvgb;

extern "C" {

int tvgb_build_neighbors2d(int w, float sigma1, float sigma2, unsigned power, unsigned samples, int stick, int plate,
                           void* out, int* count) {
    TVGB_CHECK_ARG(count, "tvgb_build_neighbors2d: count is NULL");
    TVGB_CHECK_ARG(w >= 0, "tvgb_build_neighbors2d: w must be >= 0");
    *count = build_table(w, sigma1, sigma2, power, samples, stick != 0, plate != 0, static_cast<Nb2*>(out));
    return TVGB_OK;
}

static int check2(const float* t_out, const float* t_in, float s1, unsigned w, const char* fn) {
    TVGB_CHECK_ARG(t_out && t_in, "%s: NULL field pointer", fn);
    TVGB_CHECK_ARG(s1 > 0.0f, "%s: sigma1 must be > 0", fn);
    TVGB_CHECK_ARG(w >= 1 && (w % 2) == 1, "%s: window w must be a positive odd integer (got %u)", fn, w);
    TVGB_CHECK_ARG(w <= 1025, "%s: window w = %u too large", fn, w);
    return TVGB_OK;
}

int tvgb_tensorvote(float* t_out, const float* t_in, float sigma1, float sigma2, int power, unsigned w, unsigned shape0,
                    unsigned shape1, int stick, int plate, unsigned samples, int is_atv, void* stream) {
    TVGB_TRY(check2(t_out, t_in, sigma1, w, "tvgb_tensorvote"));
    if (size_t(shape0) * shape1 == 0) return TVGB_OK;
    return vote2_impl(t_out, t_in, nullptr, 0, sigma1, sigma2, power, w, shape0, shape1, stick != 0, plate != 0,
                      samples, is_atv != 0, as_stream(stream));
}

int tvgb_tensorvote_prebuilt(float* t_out, const float* t_in, const void* host_nb, int nb_count, float sigma1,
                             float sigma2, int power, unsigned w, unsigned shape0, unsigned shape1, int stick, int plate,
                             unsigned samples, void* stream) {
    TVGB_TRY(check2(t_out, t_in, sigma1, w, "tvgb_tensorvote_prebuilt"));
    TVGB_CHECK_ARG(nb_count >= 0 && (nb_count == 0 || host_nb), "tvgb_tensorvote_prebuilt: bad neighbour table");
    if (size_t(shape0) * shape1 == 0) return TVGB_OK;
    if (nb_count == 0) {   // nothing to vote with: zeros, like a kernel with nb_count = 0
        const size_t n = size_t(shape0) * shape1;
        cudaStream_t st = as_stream(stream);
        DevArray dout;
        TVGB_TRY(dout.out(t_out, n * 16, st, true));
        TVGB_TRY(dout.finish());
        return sync_if(dout.owned, st);
    }
    return vote2_impl(t_out, t_in, static_cast<const Nb2*>(host_nb), nb_count, sigma1, sigma2, power, w, shape0, shape1,
                      stick != 0, plate != 0, samples, false, as_stream(stream));
}

// Parameter sweep of the TK vote (the objective evaluations of tiralib's
// optimize_tk, python/tira/tensors_lib/optimize.py:256-279): K parameter
// sets (sigma1, sigma2, power) against one input field and one target field
// G.  The input is solved once; each set gets its window
// (optimize.py:_w_from_sigma), its Neighbor2D table, one vote and the SIMF of
// G against the voted field (metrics.py:37).  simf[k] receives it; t_out, if
// given, receives the K voted fields.
int tvgb_tensorvote_sweep(const float* t_in, const float* G, unsigned shape0, unsigned shape1, const double* params,
                          int K, unsigned samples, int plate, double* simf, float* t_out, void* stream) {
    TVGB_CHECK_ARG(t_in && G && params && simf, "tvgb_tensorvote_sweep: NULL pointer");
    TVGB_CHECK_ARG(K >= 0, "tvgb_tensorvote_sweep: K must be >= 0");
    for (int k = 0; k < K; ++k) {
        TVGB_CHECK_ARG(params[3 * k] > 0.0 && params[3 * k + 1] >= 0.0 && params[3 * k + 2] >= 1.0 &&
                           params[3 * k] < 1e4 && params[3 * k + 1] < 1e4 && params[3 * k + 2] < 1e4,
                       "tvgb_tensorvote_sweep: parameter set %d out of range", k);
    }
    const size_t n = size_t(shape0) * shape1;
    if (K == 0) return TVGB_OK;
    if (n == 0) { for (int k = 0; k < K; ++k) simf[k] = 0.0; return TVGB_OK; }
    cudaStream_t st = as_stream(stream);
    DevArray din, dG, dout;
    TVGB_TRY(din.in(t_in, n * 16, st));
    TVGB_TRY(dG.in(G, n * 16, st));
    if (t_out) TVGB_TRY(dout.out(t_out, size_t(K) * n * 16, st));
    TVGB_CHECK_ARG(reinterpret_cast<uintptr_t>(din.dev) % 16 == 0 && reinterpret_cast<uintptr_t>(dG.dev) % 16 == 0 &&
                       reinterpret_cast<uintptr_t>(dout.dev) % 16 == 0,
                   "tvgb_tensorvote_sweep: fields must be 16-byte aligned");
    Scratch sv, sb, sacc;
    TVGB_TRY(sv.alloc(n * 16, st));
    if (!t_out) TVGB_TRY(sb.alloc(n * 16, st));
    TVGB_TRY(sacc.alloc(size_t(K) * 3 * sizeof(double), st));
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    size_t blocks = (n + 255) / 256;
    if (blocks > size_t(sms) * 16) blocks = size_t(sms) * 16;
    {
        KernelTimer kt_("k_prep2", st);
        k_prep2<<<unsigned(blocks ? blocks : 1), 256, 0, st>>>(din.get<float4>(), n, sv.get<float4>(), nullptr);
        kt_.stop();
    }
    TVGB_LAUNCHED();
    for (int k = 0; k < K; ++k) {
        const double s1d = params[3 * k], s2d = params[3 * k + 1];
        const int pw = std::max(1, int(params[3 * k + 2]));
        const double sm = std::max(s1d, s2d);
        int w = 2 * int(3.0 * sm) + 1;        // optimize.py:9-15
        if (w < 3) w = 3;
        if (w % 2 == 0) w += 1;
        float4* B = t_out ? dout.get<float4>() + size_t(k) * n : sb.get<float4>();
        TVGB_TRY(vote2_tk_launch(sv.get<float4>(), nullptr, 0, float(s1d), float(s2d), pw, unsigned(w), shape0, shape1,
                                 true, plate != 0, samples, B, st));
        TVGB_TRY(simf2_device(dG.get<float4>(), B, n, sacc.get<double>() + 3 * k, st));
    }
    std::vector<double> acc(size_t(K) * 3);
    TVGB_CUDA(cudaMemcpyAsync(acc.data(), sacc.get<double>(), acc.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    TVGB_TRY(dout.finish());
    TVGB_CUDA(cudaStreamSynchronize(st));
    for (int k = 0; k < K; ++k) simf[k] = acc[3 * k + 2] / double(n);
    return TVGB_OK;
}

}  // extern "C"
