// Adjoint (reverse-mode derivative) of the fused flocking step.
//
// The forward step of a plain flock (separation, alignment, cohesion in the
// scenario's order, then integration; SteerFor*CUDAKernel.cu and
// UpdateCUDAKernel.cu:78-123) maps each agent's position p and velocity
// v = heading * speed to
//   S  = sum_b w_b F_b,             F_b = normalize(q_b)
//        q_sep = mean over members of -(p_j - p) / |p_j - p|^2
//        q_coh = mean over members of p_j  - p
//        q_ali = mean over members of d_j  - d,   d = v / |v|
//   v' = trunc(v + trunc(S, maxForce) / mass * dt, maxSpeed)
//   p' = p + v' * dt
// where trunc(x, L) = x if |x| <= L else x L / |x|.  The KNN lists and the
// neighbourhood memberships (inBoidNeighborhood) are piecewise constant and
// are frozen at the forward pass's values: the recorded lists are reused and
// the memberships are recomputed from the recorded state with the forward
// kernels' exact FP32 operations, so both match the forward pass bit for bit.
//
// One thread per agent re-evaluates its forward quantities, then pushes the
// adjoint back:
//   g_v'  = lambda_v' + dt lambda_p'
//   g_u   = J_trunc(u, maxSpeed)^T g_v'            (u = v + a dt)
//   g_S   = J_trunc(S, maxForce)^T (dt g_u / mass)
//   dL/dw_b += g_S . F_b ;  g_q_b = (I - F_b F_b^T) w_b g_S / |q_b|
// and writes the neighbour terms of each KNN edge (agent i, rank r) to its
// own slot:
//   separation  g_o = (2 o (o . g) - |o|^2 g) / |o|^4,  g = g_q / n_members
//   cohesion    g_q / n_members to each member's position
//   alignment   g_q / n_members to each member's heading, turned into a
//               velocity adjoint with (I - d d^T) / |v|
// A kernel with one thread per edge files every edge in its target's bucket
// (kBucket slots per agent taken with an integer atomic, an overflow list
// past that).  The gather gives each agent the sum of its own terms and of
// the terms of every edge that points at it, added in ascending edge order
// whatever order the bucket was filled in.  No float atomics: two backward passes give the same
// gradients bit for bit.
// The derivative of the world wrap is the identity.
#include <cfloat>
#include <climits>

#include "gs_behaviours.cuh"
#include "gs_launch.h"

namespace gs {
namespace {

constexpr unsigned kAdjBlock = 256;

__device__ __forceinline__ V3 trunc_vjp(V3 x, float max_len, V3 g) {
    const float len_sq = dot(x, x);
    if (len_sq <= max_len * max_len) return g;
    const float len = sqrtf(len_sq);
    const V3 xh = dvd(x, len);
    return mul(sub(g, mul(xh, dot(xh, g))), max_len / len);
}

// (I - F F^T) g / |q|, the vector-Jacobian product of F = q / |q|
__device__ __forceinline__ V3 normalize_vjp(V3 F, float qlen, V3 g) {
    return dvd(sub(g, mul(F, dot(F, g))), qlen);
}

__device__ __forceinline__ float4 f4z(V3 v) { return make_float4(v.x, v.y, v.z, 0.f); }

struct Beh {
    bool on;
    V3 F, gq;  // unit direction and the adjoint of its argument q
    float qlen, inv_n;
};

__global__ void __launch_bounds__(kAdjBlock) k_flock_adjoint(AdjointLaunch A, StepDev p) {
    const unsigned i = blockIdx.x * blockDim.x + threadIdx.x;
    float gw[3] = {0.f, 0.f, 0.f};  // separation, alignment, cohesion
    if (i < A.n) {
        const float4 P = A.pos[i], D = A.dir[i];
        const V3 pos = v3(P), dir = v3(D);
        const float speed = P.w;
        const FlockParams fs = flock_params(p.sep, p.sep_dsq), fa = flock_params(p.ali, p.ali_dsq),
                          fc = flock_params(p.coh, p.coh_dsq);
        const unsigned* nb = A.knn + size_t(i) * A.k;

        // forward: memberships (same operands and tests as the fused kernel)
        FlockAcc as, aa, ac;
        flock_init(as);
        flock_init(aa);
        flock_init(ac);
        unsigned ms = 0, ma = 0, mc = 0;
        for (unsigned r = 0; r < A.k; ++r) {
            const unsigned j = nb[r];
            if (j >= A.n) break;
            const V3 bpos = v3(A.pos[j]);
            const V3 offset = sub(bpos, pos);
            const float dsq = dot(offset, offset);
            const float d = sqrtf(dsq);
            const bool ang_s = (p.need & NEED_SEP) && !(d < fs.min_d) && !(d > fs.max_d);
            const bool ang_a = (p.need & NEED_ALI) && !(d < fa.min_d) && !(d > fa.max_d);
            const bool ang_c = (p.need & NEED_COH) && !(d < fc.min_d) && !(d > fc.max_d);
            float fwd = 0.f;
            if (ang_s || ang_a || ang_c) fwd = dot(dir, dvd(offset, d));
            if ((p.need & NEED_SEP) && ((d < fs.min_d) || (ang_s && fwd > fs.cos_max))) {
                as.sum = add(as.sum, dvd(offset, -dsq));
                as.n++;
                ms |= 1u << r;
            }
            if ((p.need & NEED_ALI) && ((d < fa.min_d) || (ang_a && fwd > fa.cos_max))) {
                aa.sum = add(aa.sum, v3(A.dir[j]));
                aa.n++;
                ma |= 1u << r;
            }
            if ((p.need & NEED_COH) && ((d < fc.min_d) || (ang_c && fwd > fc.cos_max))) {
                ac.sum = add(ac.sum, bpos);
                ac.n++;
                mc |= 1u << r;
            }
        }
        // forward: behaviours in order (flock_finish), steering, integration
        Beh hs{}, ha{}, hc{};  // separation, alignment, cohesion
        unsigned applied = 0;
        V3 steer = v3(0.f, 0.f, 0.f);
        auto finish = [&](int kind, const FlockAcc& acc, const FlockParams& fp, Beh& h) {
            if (applied & fp.mask) return;
            V3 r = acc.sum;
            if (acc.n > 0) {
                const V3 mean = dvd(acc.sum, float(acc.n));
                const V3 q = kind == 0 ? mean : kind == 1 ? sub(mean, dir) : sub(mean, pos);
                h.qlen = length(q);
                h.F = normalize(q);
                h.on = h.qlen > 0.f;
                h.inv_n = 1.f / float(acc.n);
                r = h.F;
            }
            r = mul(r, fp.w);
            const unsigned bit = kind == 0 ? SEPARATION_BIT : kind == 1 ? ALIGNMENT_BIT : COHESION_BIT;
            if (!is_zero(r)) applied |= bit;
            steer = add(r, steer);
        };
#pragma unroll
        for (unsigned o = 0; o < 8; ++o) {
            if (o >= p.n_order) continue;
            switch (p.order[o]) {
                case GS_B_SEPARATION: finish(0, as, fs, hs); break;
                case GS_B_ALIGNMENT: finish(1, aa, fa, ha); break;
                case GS_B_COHESION: finish(2, ac, fc, hc); break;
                default: break;
            }
        }
        const float max_force = A.max_force[i], max_speed = A.max_speed[i], mass = A.mass[i];
        const V3 st = truncate_length(steer, max_force);
        const V3 u = add(mul(dir, speed), mul(dvd(st, mass), p.dt));

        // backward
        const V3 gp1 = v3(A.lp_in[i]), gv1 = v3(A.lv_in[i]);
        A.lp_in[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        A.lv_in[i] = make_float4(0.f, 0.f, 0.f, 0.f);
        const V3 gu = trunc_vjp(u, max_speed, add(gv1, mul(gp1, p.dt)));
        const V3 gS = trunc_vjp(steer, max_force, dvd(mul(gu, p.dt), mass));
        V3 own_p = gp1, own_v = gu, own_d = v3(0.f, 0.f, 0.f);
        auto back = [&](Beh& h, float w, float& gwb) {
            if (!h.on) return;
            gwb = dot(gS, h.F);
            h.gq = normalize_vjp(h.F, h.qlen, mul(gS, w));
        };
        back(hs, fs.w, gw[0]);
        back(ha, fa.w, gw[1]);
        back(hc, fc.w, gw[2]);
        if (hc.on) own_p = sub(own_p, hc.gq);
        if (ha.on) own_d = sub(own_d, ha.gq);
        const V3 g_sep = hs.on ? mul(hs.gq, hs.inv_n) : v3(0.f, 0.f, 0.f);
        const V3 g_coh = hc.on ? mul(hc.gq, hc.inv_n) : v3(0.f, 0.f, 0.f);
        const V3 g_ali = ha.on ? mul(ha.gq, ha.inv_n) : v3(0.f, 0.f, 0.f);
        const unsigned m_sep = hs.on ? ms : 0u, m_ali = ha.on ? ma : 0u,
                       m_coh = hc.on ? mc : 0u;
        // every listed edge gets its slot written (zero where it adds nothing)
        for (unsigned r = 0; r < A.k; ++r) {
            const unsigned j = nb[r];
            if (j >= A.n) break;
            V3 gpj = v3(0.f, 0.f, 0.f), gvj = v3(0.f, 0.f, 0.f);
            if ((m_sep >> r) & 1u) {
                const V3 o = sub(v3(A.pos[j]), pos);
                const float oo = dot(o, o);
                const V3 go = dvd(sub(mul(o, 2.f * dot(o, g_sep)), mul(g_sep, oo)), oo * oo);
                gpj = add(gpj, go);
                own_p = sub(own_p, go);
            }
            if ((m_coh >> r) & 1u) gpj = add(gpj, g_coh);
            if ((m_ali >> r) & 1u) {
                const float4 Pj = A.pos[j];
                const V3 dj = v3(A.dir[j]);
                if (Pj.w > 0.f) gvj = dvd(sub(g_ali, mul(dj, dot(dj, g_ali))), Pj.w);
            }
            const unsigned e = i * A.k + r;
            A.edge_p[e] = f4z(gpj);
            A.edge_v[e] = f4z(gvj);
        }
        if (speed > 0.f) own_v = add(own_v, dvd(sub(own_d, mul(dir, dot(dir, own_d))), speed));
        A.own_p[i] = f4z(own_p);
        A.own_v[i] = f4z(own_v);
    }
    // per-block sums of the weight adjoints (fixed order: deterministic)
    __shared__ float red[3][kAdjBlock / 32];
#pragma unroll
    for (int b = 0; b < 3; ++b) {
        float v = gw[b];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) red[b][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        float v = 0.f;
        for (unsigned w = 0; w < blockDim.x / 32; ++w) v += red[threadIdx.x][w];
        A.wpart[blockIdx.x * 4 + threadIdx.x] += v;
    }
}

// Files edge e = i * k + r in the bucket of its target knn[e].
__global__ void __launch_bounds__(kAdjBlock) k_bucket_edges(AdjointLaunch A) {
    const unsigned e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= A.n * A.k) return;
    const unsigned j = A.knn[e];
    if (j >= A.n) return;
    const unsigned slot = atomicAdd(A.fill + j, 1u);
    if (slot < kBucket) {
        A.bucket[size_t(j) * kBucket + slot] = e;
    } else {
        const unsigned o = atomicAdd(A.fill + A.n, 1u);
        A.ovf[2 * size_t(o)] = j;
        A.ovf[2 * size_t(o) + 1] = e;
    }
}

// Agent j's input adjoints: its own terms, then the terms of the edges into
// it in ascending edge order, added to lp_out / lv_out.  Up to kBucket edges
// (in-degrees stay near k) are sorted in a local array; an agent with more
// walks its bucket and the overflow list by repeated minimum search.
__global__ void __launch_bounds__(kAdjBlock) k_adjoint_gather(AdjointLaunch A) {
    const unsigned j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= A.n) return;
    const unsigned deg = A.fill[j];
    const unsigned* bk = A.bucket + size_t(j) * kBucket;
    V3 gp = v3(A.own_p[j]), gv = v3(A.own_v[j]);
    auto add_edge = [&](unsigned e) {
        gp = add(gp, v3(A.edge_p[e]));
        gv = add(gv, v3(A.edge_v[e]));
    };
    if (deg <= kBucket) {
        unsigned es[kBucket];
        for (unsigned t = 0; t < deg; ++t) {  // insertion sort, ascending
            const unsigned e = bk[t];
            unsigned q = t;
            while (q > 0 && es[q - 1] > e) {
                es[q] = es[q - 1];
                --q;
            }
            es[q] = e;
        }
        for (unsigned t = 0; t < deg; ++t) add_edge(es[t]);
    } else {
        const unsigned n_ovf = A.fill[A.n];
        unsigned last = 0;
        for (unsigned t = 0; t < deg; ++t) {
            unsigned best = UINT_MAX;
            for (unsigned q = 0; q < kBucket; ++q) {
                const unsigned e = bk[q];
                if ((t == 0 || e > last) && e < best) best = e;
            }
            for (unsigned q = 0; q < n_ovf; ++q) {
                if (A.ovf[2 * size_t(q)] != j) continue;
                const unsigned e = A.ovf[2 * size_t(q) + 1];
                if ((t == 0 || e > last) && e < best) best = e;
            }
            add_edge(best);
            last = best;
        }
    }
    const float4 op = A.lp_out[j], ov = A.lv_out[j];
    A.lp_out[j] = make_float4(op.x + gp.x, op.y + gp.y, op.z + gp.z, 0.f);
    A.lv_out[j] = make_float4(ov.x + gv.x, ov.y + gv.y, ov.z + gv.z, 0.f);
}

}  // namespace

unsigned adjoint_blocks(unsigned n) { return n ? (n + kAdjBlock - 1) / kAdjBlock : 1u; }

size_t adjoint_scratch_bytes(unsigned n, unsigned k) {
    const size_t nk = size_t(n) * k;
    return nk * 32 + size_t(n) * 32 + (size_t(n) + 1) * 4 + size_t(n) * kBucket * 4 + nk * 8 +
           6 * 256;
}

// Carves the scratch of one adjoint step out of `base` (adjoint_scratch_bytes).
void adjoint_scratch_bind(AdjointLaunch& A, void* base, unsigned n, unsigned k) {
    auto align = [](size_t x) { return (x + 255) & ~size_t(255); };
    char* b = static_cast<char*>(base);
    const size_t nk = size_t(n) * k;
    size_t o = 0;
    A.edge_p = reinterpret_cast<float4*>(b + o);
    o = align(o + nk * 16);
    A.edge_v = reinterpret_cast<float4*>(b + o);
    o = align(o + nk * 16);
    A.own_p = reinterpret_cast<float4*>(b + o);
    o = align(o + size_t(n) * 16);
    A.own_v = reinterpret_cast<float4*>(b + o);
    o = align(o + size_t(n) * 16);
    A.fill = reinterpret_cast<unsigned*>(b + o);
    o = align(o + (size_t(n) + 1) * 4);
    A.bucket = reinterpret_cast<unsigned*>(b + o);
    o = align(o + size_t(n) * kBucket * 4);
    A.ovf = reinterpret_cast<unsigned*>(b + o);
}

gs_status launch_flock_adjoint(const AdjointLaunch& A, const StepDev& p, cudaStream_t st) {
    if (A.k == 0 || A.k > 32) return fail(GS_ERR_INVALID_ARG, "adjoint needs 1 <= k <= 32");
    if (A.n == 0) return GS_OK;
    if (size_t(A.n) * A.k > 0xffffffffull) return fail(GS_ERR_INVALID_ARG, "too many KNN edges");
    // bucket fill counts and the overflow count start at zero
    GS_CUDA(cudaMemsetAsync(A.fill, 0, (size_t(A.n) + 1) * 4, st));
    k_bucket_edges<<<adjoint_blocks(A.n * A.k), kAdjBlock, 0, st>>>(A);
    // each agent's terms and its edges' terms, then the gather
    k_flock_adjoint<<<adjoint_blocks(A.n), kAdjBlock, 0, st>>>(A, p);
    k_adjoint_gather<<<adjoint_blocks(A.n), kAdjBlock, 0, st>>>(A);
    GS_LAUNCHED("flock_adjoint");
    return GS_OK;
}

}  // namespace gs
