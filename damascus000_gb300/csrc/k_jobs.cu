// Multi-job kernels: register-resident NTTs, column MACs, the inverse-NTT + CRT
// finish, coefficient-domain folds and the BLAKE3 expansion, each taking a list
// of jobs so that one launch covers the same stage of many requests.
#include <cuda_runtime.h>

#include "dm_blake3.cuh"
#include "dm_jobs.cuh"
#include "dm_ntt.cuh"
#include "dm_tables.h"

namespace dm {

namespace {

template <class J>
struct JobList {
    J j[kMaxJobs];
    int n;
};

// Job of this CTA (jobs are sorted by cta0; at most kMaxJobs, uniform per CTA).
template <class J>
DM_D int find_job(const JobList<J>& L) {
    int k = 0;
    while (k + 1 < L.n && blockIdx.x >= L.j[k + 1].cta0) ++k;
    return k;
}

DM_D fq ldq(const uint4* p, uint64_t i) {
    const uint4 v = p[i];
    return fq{{v.x, v.y, v.z, v.w}};
}
DM_D void stq(uint4* p, uint64_t i, const fq& a) { p[i] = make_uint4(a.w[0], a.w[1], a.w[2], a.w[3]); }

// ================================================================ forward NTT
template <int L>
struct NttShape {
    static constexpr int T = 1 << (L - 4);                                  // threads per row
    static constexpr int PR = (L >= 12) ? 4 : 8;                             // primes per CTA
    static constexpr int P = (PR * T >= 256) ? 1 : 256 / (PR * T);           // polynomials per CTA
    static constexpr int THREADS = P * PR * T;
    static constexpr int PASSES = (L + 3) / 4;
    static constexpr int SPLIT = 8 / PR;                                     // CTAs per polynomial group
    static constexpr size_t SMEM = (size_t)P * PR * (1u << L) * sizeof(uint32_t);
};

template <int L>
__global__ void __launch_bounds__(NttShape<L>::THREADS)
    ntt_fwd_jobs_kernel(JobList<NttJob> J, PrimeConsts pc, const uint32_t* __restrict__ zeta,
                        const uint32_t* __restrict__ zetap) {
    using S = NttShape<L>;
    extern __shared__ __align__(16) uint32_t sm[];
    const NttJob jb = J.j[find_job(J)];
    const uint32_t lcta = blockIdx.x - jb.cta0;
    const uint32_t half = (S::SPLIT == 2) ? (lcta & 1u) : 0u;
    const uint64_t poly = (uint64_t)(lcta / S::SPLIT) * S::P + threadIdx.x / (S::T * S::PR);
    const uint32_t t = threadIdx.x % S::T;
    const uint32_t row = threadIdx.x / S::T;
    const uint32_t pi = half * S::PR + row % S::PR;
    const bool active = poly < jb.npolys;
    const uint32_t p = pc.p[pi];
    const uint32_t* zt = zeta + pi * kMaxRing;
    const uint32_t* ztp = zetap + pi * kMaxRing;
    uint32_t a[kNttE];
    if (active) {
        const uint4* src = jb.src + (poly << L);
#pragma unroll
        for (int r = 0; r < kNttE; ++r) a[r] = residue_lazy(ldq(src, ntt_place(L, 0, t, r)), pc, pi);
    } else {
#pragma unroll
        for (int r = 0; r < kNttE; ++r) a[r] = 0;
    }
    uint32_t* srow = sm + row * (1u << L);
#pragma unroll
    for (int pass = 0; pass < S::PASSES; ++pass) {
        ntt_fwd_pass_lazy(a, L, pass, t, zt, ztp, p);
        if (pass + 1 < S::PASSES) {
#pragma unroll
            for (int r = 0; r < kNttE; ++r) srow[ntt_swz(ntt_place(L, pass, t, r))] = a[r];
            __syncthreads();
#pragma unroll
            for (int r = 0; r < kNttE; ++r) a[r] = srow[ntt_swz(ntt_place(L, pass + 1, t, r))];
            __syncthreads();
        }
    }
    if (active) {
#pragma unroll
        for (int r = 0; r < kNttE; ++r) a[r] = normalize_lazy(a[r], pc, pi);
        uint4* dst = reinterpret_cast<uint4*>(jb.dst + ((poly * kPrimes + pi) << L) + t * kNttE);
        dst[0] = make_uint4(a[0], a[1], a[2], a[3]);
        dst[1] = make_uint4(a[4], a[5], a[6], a[7]);
        dst[2] = make_uint4(a[8], a[9], a[10], a[11]);
        dst[3] = make_uint4(a[12], a[13], a[14], a[15]);
    }
}

// Rings smaller than 16: one thread per (polynomial, prime), all in registers.
template <int L>
__global__ void ntt_fwd_small_kernel(JobList<NttJob> J, PrimeConsts pc, const uint32_t* __restrict__ zeta,
                                     const uint32_t* __restrict__ zetap) {
    constexpr int s = 1 << L;
    const NttJob jb = J.j[find_job(J)];
    const uint64_t item = (uint64_t)(blockIdx.x - jb.cta0) * blockDim.x + threadIdx.x;
    const uint64_t poly = item >> 3;
    const uint32_t pi = (uint32_t)(item & 7u);
    if (poly >= jb.npolys) return;
    const uint32_t p = pc.p[pi];
    const uint32_t* zt = zeta + pi * kMaxRing;
    const uint32_t* ztp = zetap + pi * kMaxRing;
    uint32_t a[s];
#pragma unroll
    for (int c = 0; c < s; ++c) a[c] = residue_fast(ldq(jb.src + (poly << L), c), pc, pi);
#pragma unroll
    for (int st = 0; st < L; ++st) {
        const int len = s >> (st + 1);
#pragma unroll
        for (int j = 0; j < s; ++j) {
            if (j & len) continue;
            const uint32_t k = (1u << st) + (uint32_t)(j >> (L - st));
            const uint32_t v = mont_tw(a[j + len], zt[k], ztp[k], p);
            const uint32_t u = a[j];
            a[j] = add_mod(u, v, p);
            a[j + len] = sub_mod(u, v, p);
        }
    }
#pragma unroll
    for (int c = 0; c < s; ++c) jb.dst[((poly * kPrimes + pi) << L) + c] = a[c];
}

// ================================================================ MAC
constexpr int kMacThreads = 128;

DM_D uint32_t slot_block_count(uint32_t s) { return (s + kMacThreads - 1) / kMacThreads; }

// grid: per job, nblk * 64 * parts CTAs; CTA -> (part, kp, slot block).
__global__ void __launch_bounds__(kMacThreads) mac_jobs_kernel(JobList<MacJobX> J, uint32_t L, PrimeConsts pc) {
    const MacJobX jb = J.j[find_job(J)];
    const uint32_t s = 1u << L;
    const uint32_t nblk = slot_block_count(s);
    uint32_t c = blockIdx.x - jb.cta0;
    const uint32_t blk = c % nblk;
    c /= nblk;
    const uint32_t kp = c % 64;
    const uint32_t part = c / 64;
    const uint32_t slot = blk * kMacThreads + threadIdx.x;
    if (slot >= s) return;
    const uint32_t k = kp >> 3, pi = kp & 7u;
    const uint32_t i0 = (uint32_t)((uint64_t)jb.count * part / jb.parts);
    const uint32_t i1 = (uint32_t)((uint64_t)jb.count * (part + 1) / jb.parts);
    const uint32_t p = pc.p[pi], pv = pc.pinv[pi];
    const uint64_t gstride = (uint64_t)kRank * kPrimes << L;  // one generator vector
    const uint64_t mstride = (uint64_t)kPrimes << L;
    const uint32_t* g = jb.G + ((((uint64_t)jb.g_base * kRank + k) * kPrimes + pi) << L) + slot;
    const uint32_t* m = jb.M + (((uint64_t)jb.m_base * kPrimes + pi) << L) + slot;
    uint64_t acc0 = 0, acc1 = 0;
    uint32_t i = i0;
    for (; i + 4 <= i1; i += 4) {
        const uint32_t g0 = __ldg(g + i * gstride), g1 = __ldg(g + (i + 1) * gstride);
        const uint32_t g2 = __ldg(g + (i + 2) * gstride), g3 = __ldg(g + (i + 3) * gstride);
        const uint32_t m0 = __ldg(m + i * mstride), m1 = __ldg(m + (i + 1) * mstride);
        const uint32_t m2 = __ldg(m + (i + 2) * mstride), m3 = __ldg(m + (i + 3) * mstride);
        acc0 += mont_mul(g0, m0, p, pv);
        acc1 += mont_mul(g1, m1, p, pv);
        acc0 += mont_mul(g2, m2, p, pv);
        acc1 += mont_mul(g3, m3, p, pv);
    }
    for (; i < i1; ++i) acc0 += mont_mul(__ldg(g + i * gstride), __ldg(m + i * mstride), p, pv);
    jb.out0[(((uint64_t)part * 64 + kp) << L) + slot] = reduce_u64(acc0 + acc1, p, pv, pc.r1[pi], pc.r2[pi]);
}

// Triple MAC over h = count column pairs (i, i + h): one read of every generator
// column gives the full sum (out0), L = sum G[i+h] M[i] (out1) and
// R = sum G[i] M[i+h] (out2).
__global__ void __launch_bounds__(kMacThreads) mac_triple_jobs_kernel(JobList<MacJobX> J, uint32_t L, PrimeConsts pc) {
    const MacJobX jb = J.j[find_job(J)];
    const uint32_t s = 1u << L;
    const uint32_t nblk = slot_block_count(s);
    uint32_t c = blockIdx.x - jb.cta0;
    const uint32_t blk = c % nblk;
    c /= nblk;
    const uint32_t kp = c % 64;
    const uint32_t part = c / 64;
    const uint32_t slot = blk * kMacThreads + threadIdx.x;
    if (slot >= s) return;
    const uint32_t k = kp >> 3, pi = kp & 7u;
    const uint32_t h = jb.count;
    const uint32_t i0 = (uint32_t)((uint64_t)h * part / jb.parts);
    const uint32_t i1 = (uint32_t)((uint64_t)h * (part + 1) / jb.parts);
    const uint32_t p = pc.p[pi], pv = pc.pinv[pi];
    const uint64_t gstride = (uint64_t)kRank * kPrimes << L;
    const uint64_t mstride = (uint64_t)kPrimes << L;
    const uint32_t* g = jb.G + ((((uint64_t)k) * kPrimes + pi) << L) + slot;
    const uint32_t* m = jb.M + (((uint64_t)pi) << L) + slot;
    const uint64_t gh = (uint64_t)h * gstride, mh = (uint64_t)h * mstride;
    uint64_t ac = 0, al = 0, ar = 0;
    for (uint32_t i = i0; i < i1; ++i) {
        const uint32_t gl = __ldg(g + i * gstride), gr = __ldg(g + i * gstride + gh);
        const uint32_t ml = __ldg(m + i * mstride), mr = __ldg(m + i * mstride + mh);
        ac += mont_mul(gl, ml, p, pv);
        ac += mont_mul(gr, mr, p, pv);
        al += mont_mul(gr, ml, p, pv);
        ar += mont_mul(gl, mr, p, pv);
    }
    const uint32_t r1 = pc.r1[pi], r2 = pc.r2[pi];
    const uint64_t o = (((uint64_t)part * 64 + kp) << L) + slot;
    jb.out0[o] = reduce_u64(ac, p, pv, r1, r2);
    jb.out1[o] = reduce_u64(al, p, pv, r1, r2);
    jb.out2[o] = reduce_u64(ar, p, pv, r1, r2);
}

// Split MAC: thread per slot pair of ring 2^L (L >= 1).
__global__ void __launch_bounds__(kMacThreads) mac_split_jobs_kernel(JobList<MacJobX> J, uint32_t L, PrimeConsts pc) {
    const MacJobX jb = J.j[find_job(J)];
    const uint32_t h = 1u << (L - 1);
    const uint32_t nblk = slot_block_count(h);
    uint32_t c = blockIdx.x - jb.cta0;
    const uint32_t blk = c % nblk;
    c /= nblk;
    const uint32_t kp = c % 64;
    const uint32_t part = c / 64;
    const uint32_t i2 = blk * kMacThreads + threadIdx.x;
    if (i2 >= h) return;
    const uint32_t k = kp >> 3, pi = kp & 7u;
    const uint32_t i0 = (uint32_t)((uint64_t)jb.count * part / jb.parts);
    const uint32_t i1 = (uint32_t)((uint64_t)jb.count * (part + 1) / jb.parts);
    const uint32_t p = pc.p[pi], pv = pc.pinv[pi];
    const uint64_t gstride = (uint64_t)kRank * kPrimes << L;
    const uint64_t mstride = (uint64_t)kPrimes << L;
    const uint32_t* g = jb.G + ((((uint64_t)jb.g_base * kRank + k) * kPrimes + pi) << L) + 2 * i2;
    const uint32_t* m = jb.M + (((uint64_t)jb.m_base * kPrimes + pi) << L) + 2 * i2;
    uint64_t a0 = 0, a1 = 0, al = 0, ar = 0;
    for (uint32_t i = i0; i < i1; ++i) {
        const uint2 gv = __ldg(reinterpret_cast<const uint2*>(g + i * gstride));
        const uint2 mv = __ldg(reinterpret_cast<const uint2*>(m + i * mstride));
        a0 += mont_mul(gv.x, mv.x, p, pv);
        a1 += mont_mul(gv.y, mv.y, p, pv);
        al += mont_mul(sub_mod(gv.x, gv.y, p), add_mod(mv.x, mv.y, p), p, pv);
        ar += mont_mul(add_mod(gv.x, gv.y, p), sub_mod(mv.x, mv.y, p), p, pv);
    }
    const uint32_t r1 = pc.r1[pi], r2 = pc.r2[pi];
    *reinterpret_cast<uint2*>(jb.out0 + (((uint64_t)part * 64 + kp) << L) + 2 * i2) =
        make_uint2(reduce_u64(a0, p, pv, r1, r2), reduce_u64(a1, p, pv, r1, r2));
    jb.out1[(((uint64_t)part * 64 + kp) << (L - 1)) + i2] = reduce_u64(al, p, pv, r1, r2);
    jb.out2[(((uint64_t)part * 64 + kp) << (L - 1)) + i2] = reduce_u64(ar, p, pv, r1, r2);
}

// ================================================================ finish
struct FinishConsts {
    uint32_t f[kPrimes], fp[kPrimes];  // final inverse-NTT scale (Montgomery form) and its product with p^-1
};

template <int L>
struct FinShape {
    static constexpr int T = 1 << (L - 4);
    static constexpr int THREADS = kPrimes * T;  // one CTA per (job, coordinate)
    static constexpr int PASSES = (L + 3) / 4;
    static constexpr size_t SMEM = (size_t)kPrimes * (1u << L) * sizeof(uint32_t);
};

// grid: (8 coordinates, njobs).  Sums the column partials, applies the split
// scale (w_i or w_i^-1, the 1/4 lives in the final scale), inverse-transforms,
// recombines the eight residues of every slot by Garner CRT into Z_q and
// optionally compares with the expected commitment.
template <int L>
__global__ void __launch_bounds__(FinShape<L>::THREADS)
    finish_jobs_kernel(JobList<FinishJobX> J, PrimeConsts pc, CrtConsts cc, FinishConsts plain, FinishConsts split,
                       const uint32_t* __restrict__ zeta, const uint32_t* __restrict__ zetap,
                       const uint32_t* __restrict__ zinv, const uint32_t* __restrict__ zinvp) {
    using S = FinShape<L>;
    constexpr uint32_t s = 1u << L;
    extern __shared__ __align__(16) uint32_t sm[];
    const FinishJobX jb = J.j[blockIdx.y];
    const uint32_t k = blockIdx.x;
    const uint32_t t = threadIdx.x % S::T;
    const uint32_t pi = threadIdx.x / S::T;
    const uint32_t p = pc.p[pi], pv = pc.pinv[pi];
    uint32_t a[kNttE];
#pragma unroll
    for (int r = 0; r < kNttE; ++r) a[r] = 0;
    for (uint32_t part = 0; part < jb.parts; ++part) {
        const uint4* src = reinterpret_cast<const uint4*>(jb.partials + (((uint64_t)part * 64 + k * 8 + pi) << L) +
                                                          t * kNttE);
#pragma unroll
        for (int q4 = 0; q4 < 4; ++q4) {
            const uint4 v = src[q4];
            a[4 * q4] = add_mod(a[4 * q4], v.x, p);
            a[4 * q4 + 1] = add_mod(a[4 * q4 + 1], v.y, p);
            a[4 * q4 + 2] = add_mod(a[4 * q4 + 2], v.z, p);
            a[4 * q4 + 3] = add_mod(a[4 * q4 + 3], v.w, p);
        }
    }
    if (jb.mode == kFinishSplitL) {
#pragma unroll
        for (int r = 0; r < kNttE; ++r) {
            const uint32_t i = s + t * kNttE + r;
            a[r] = mont_tw(a[r], zeta[pi * kMaxRing + i], zetap[pi * kMaxRing + i], p);
        }
    } else if (jb.mode == kFinishSplitR) {
#pragma unroll
        for (int r = 0; r < kNttE; ++r) {
            const uint32_t i = s + t * kNttE + r;
            a[r] = mont_tw(a[r], zinv[pi * kMaxRing + i], zinvp[pi * kMaxRing + i], p);
        }
    }
    uint32_t* srow = sm + pi * s;
    const uint32_t* zi = zinv + pi * kMaxRing;
    const uint32_t* zip = zinvp + pi * kMaxRing;
#pragma unroll
    for (int pass = S::PASSES - 1; pass >= 0; --pass) {
        ntt_inv_pass(a, L, pass, t, zi, zip, p);
        if (pass > 0) {
#pragma unroll
            for (int r = 0; r < kNttE; ++r) srow[ntt_swz(ntt_place(L, pass, t, r))] = a[r];
            __syncthreads();
#pragma unroll
            for (int r = 0; r < kNttE; ++r) a[r] = srow[ntt_swz(ntt_place(L, pass - 1, t, r))];
            __syncthreads();
        }
    }
    const FinishConsts& fc = (jb.mode == kFinishPlain) ? plain : split;
    const uint32_t f = fc.f[pi], fp = fc.fp[pi];
#pragma unroll
    for (int r = 0; r < kNttE; ++r) srow[ntt_place(L, 0, t, r)] = mont_tw(a[r], f, fp, p);
    __syncthreads();
    (void)pv;
    for (uint32_t c = threadIdx.x; c < s; c += blockDim.x) {
        uint32_t rr[kPrimes];
#pragma unroll
        for (int q = 0; q < kPrimes; ++q) rr[q] = sm[q * s + c];
        const fq v = crt_to_fq_fast(rr, pc, cc);
        const uint64_t o = ((uint64_t)k << L) + c;
        stq(jb.out, o, v);
        if (jb.expect) {
            const uint4 e = jb.expect[o];
            if (e.x != v.w[0] || e.y != v.w[1] || e.z != v.w[2] || e.w != v.w[3]) atomicOr(jb.flag, 1u);
        }
    }
}

// Rings below 16 coefficients: one thread per (job, coordinate, prime), then CRT.
template <int L>
__global__ void finish_small_kernel(JobList<FinishJobX> J, PrimeConsts pc, CrtConsts cc, FinishConsts plain,
                                    FinishConsts split, const uint32_t* __restrict__ zeta,
                                    const uint32_t* __restrict__ zetap, const uint32_t* __restrict__ zinv,
                                    const uint32_t* __restrict__ zinvp) {
    constexpr int s = 1 << L;
    __shared__ uint32_t sm[kRank][kPrimes][s];
    const FinishJobX jb = J.j[blockIdx.y];
    const uint32_t k = threadIdx.x >> 3, pi = threadIdx.x & 7u;  // 64 threads
    const uint32_t p = pc.p[pi];
    uint32_t a[s];
#pragma unroll
    for (int c = 0; c < s; ++c) {
        uint32_t acc = 0;
        for (uint32_t part = 0; part < jb.parts; ++part)
            acc = add_mod(acc, jb.partials[(((uint64_t)part * 64 + k * 8 + pi) << L) + c], p);
        if (jb.mode == kFinishSplitL) acc = mont_tw(acc, zeta[pi * kMaxRing + s + c], zetap[pi * kMaxRing + s + c], p);
        if (jb.mode == kFinishSplitR) acc = mont_tw(acc, zinv[pi * kMaxRing + s + c], zinvp[pi * kMaxRing + s + c], p);
        a[c] = acc;
    }
    const uint32_t* zi = zinv + pi * kMaxRing;
    const uint32_t* zip = zinvp + pi * kMaxRing;
#pragma unroll
    for (int st = L - 1; st >= 0; --st) {
        const int len = s >> (st + 1);
#pragma unroll
        for (int j = 0; j < s; ++j) {
            if (j & len) continue;
            const uint32_t kk = (1u << st) + (uint32_t)(j >> (L - st));
            const uint32_t u = a[j], v = a[j + len];
            a[j] = add_mod(u, v, p);
            a[j + len] = mont_tw(sub_mod(u, v, p), zi[kk], zip[kk], p);
        }
    }
    const FinishConsts& fc = (jb.mode == kFinishPlain) ? plain : split;
#pragma unroll
    for (int c = 0; c < s; ++c) sm[k][pi][c] = mont_tw(a[c], fc.f[pi], fc.fp[pi], p);
    __syncthreads();
    for (uint32_t e = threadIdx.x; e < (uint32_t)(kRank * s); e += blockDim.x) {
        const uint32_t kk = e / s, c = e % s;
        uint32_t rr[kPrimes];
#pragma unroll
        for (int q = 0; q < kPrimes; ++q) rr[q] = sm[kk][q][c];
        const fq v = crt_to_fq_fast(rr, pc, cc);
        const uint64_t o = ((uint64_t)kk << L) + c;
        stq(jb.out, o, v);
        if (jb.expect) {
            const uint4 ex = jb.expect[o];
            if (ex.x != v.w[0] || ex.y != v.w[1] || ex.z != v.w[2] || ex.w != v.w[3]) atomicOr(jb.flag, 1u);
        }
    }
}

// ================================================================ folds
constexpr int kFoldThreads = 256;
constexpr int kFoldItems = 4;  // elements per thread

__global__ void __launch_bounds__(kFoldThreads) fold_jobs_kernel(JobList<FoldJob> J) {
    const FoldJob jb = J.j[find_job(J)];
    const uint64_t base = (uint64_t)(blockIdx.x - jb.cta0) * kFoldThreads * kFoldItems + threadIdx.x;
#pragma unroll
    for (int it = 0; it < kFoldItems; ++it) {
        const uint64_t e = base + (uint64_t)it * kFoldThreads;
        if (e >= jb.n) return;
        fq out;
        switch (jb.mode) {
            case kFoldVec:
                out = fq_fma(ldq(jb.a, e), jb.x, ldq(jb.b, e));
                break;
            case kFoldPoly:
            case kFoldPolyX: {
                const uint32_t h = 1u << jb.Lout;
                const uint64_t poly = e >> jb.Lout;
                const uint32_t j = (uint32_t)(e & (h - 1));
                const uint64_t b2 = poly << (jb.Lout + 1);
                fq odd;
                if (jb.mode == kFoldPolyX)
                    odd = j == 0 ? fq_neg(ldq(jb.a, b2 + 2 * h - 1)) : ldq(jb.a, b2 + 2 * j - 1);
                else
                    odd = ldq(jb.a, b2 + 2 * j + 1);
                out = fq_fma(ldq(jb.a, b2 + 2 * j), jb.x, odd);
                break;
            }
            case kCombine:
                out = fq_add(fq_fma(ldq(jb.a, e), jb.x, ldq(jb.b, e)), fq_mul(jb.y, ldq(jb.c, e)));
                break;
            case kCombineEven: {
                const uint64_t k = e >> jb.Lout;
                const uint32_t j = (uint32_t)(e & ((1u << jb.Lout) - 1));
                const fq even = ldq(jb.a, (k << (jb.Lout + 1)) + 2 * j);
                out = fq_add(fq_fma(even, jb.x, ldq(jb.b, e)), fq_mul(jb.y, ldq(jb.c, e)));
                break;
            }
            default: {
                const uint4 v = jb.a[e];
                uint32_t r[8] = {v.x, v.y, v.z, v.w, 0, 0, 0, 0};
                out = fq_reduce8(r);
                break;
            }
        }
        stq(jb.dst, e, out);
    }
}

// ================================================================ hashing / expansion
constexpr int kGenThreads = 256;
constexpr int kGenItems = 4;

__global__ void __launch_bounds__(kGenThreads) gen_jobs_kernel(JobList<GenJob> J) {
    const GenJob jb = J.j[find_job(J)];
    const uint64_t base = (uint64_t)(blockIdx.x - jb.cta0) * kGenThreads * kGenItems + threadIdx.x;
    for (int it = 0; it < kGenItems; ++it) {
        const uint64_t e = base + (uint64_t)it * kGenThreads;
        if (e >= jb.total) return;
        const uint64_t c = e & ((1ull << jb.log_n) - 1);
        const uint64_t kk = (e >> jb.log_n) & 7u;
        const uint64_t i = e >> (jb.log_n + 3);
        uint32_t m[16], out[16];
        b3_generator_block(i, kk, c, m);
        b3_compress(jb.key, m, 0, 25, kB3ChunkStart | kB3ChunkEnd | kB3Root | kB3Keyed, out);
        stq(jb.dst, e, fq_reduce8(out));
    }
}

__global__ void __launch_bounds__(256) unpack_jobs_kernel(JobList<UnpackJob> J) {
    const UnpackJob jb = J.j[find_job(J)];
    const uint64_t j = (uint64_t)(blockIdx.x - jb.cta0) * 256 + threadIdx.x;
    if (j >= jb.total) return;
    uint32_t w[4] = {0, 0, 0, 0};
    const uint64_t off = j * kBytesPerCoeff;
    if (off < jb.len) {
        const uint64_t n = jb.len - off < (uint64_t)kBytesPerCoeff ? jb.len - off : (uint64_t)kBytesPerCoeff;
        for (uint32_t b = 0; b < n; ++b) w[b >> 2] |= (uint32_t)jb.file[off + b] << (8 * (b & 3));
    }
    jb.dst[j] = make_uint4(w[0], w[1], w[2], w[3]);
}

DM_D void load_block16(const uint8_t* p, uint32_t n, uint32_t m[16]) {
    if (n == 64 && ((reinterpret_cast<uintptr_t>(p) & 15u) == 0)) {
        const uint4* q = reinterpret_cast<const uint4*>(p);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const uint4 v = q[i];
            m[4 * i] = v.x;
            m[4 * i + 1] = v.y;
            m[4 * i + 2] = v.z;
            m[4 * i + 3] = v.w;
        }
        return;
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) m[i] = 0;
    for (uint32_t b = 0; b < n; ++b) m[b >> 2] |= (uint32_t)p[b] << (8 * (b & 3));
}

// Chunk chaining values, one thread per 1 KiB chunk (a single chunk is the root).
__global__ void __launch_bounds__(128) hash_chunk_jobs_kernel(JobList<HashJob> J) {
    const HashJob jb = J.j[find_job(J)];
    const uint64_t nchunks = jb.len == 0 ? 1 : (jb.len + kB3ChunkLen - 1) / kB3ChunkLen;
    const uint64_t c = (uint64_t)(blockIdx.x - jb.cta0) * 128 + threadIdx.x;
    if (c >= nchunks) return;
    const uint64_t off = c * kB3ChunkLen;
    const uint32_t clen = (uint32_t)(jb.len - off < kB3ChunkLen ? jb.len - off : kB3ChunkLen);
    const uint32_t nblocks = clen == 0 ? 1u : (clen + 63u) / 64u;
    uint32_t cv[8] = {DM_B3_IV0, DM_B3_IV1, DM_B3_IV2, DM_B3_IV3, DM_B3_IV4, DM_B3_IV5, DM_B3_IV6, DM_B3_IV7};
    uint32_t m[16], out[16];
    for (uint32_t b = 0; b < nblocks; ++b) {
        const uint32_t bl = clen - b * 64u < 64u ? clen - b * 64u : 64u;
        load_block16(jb.file + off + b * 64u, clen == 0 ? 0u : bl, m);
        uint32_t flags = (b == 0 ? kB3ChunkStart : 0u);
        if (b + 1 == nblocks) flags |= kB3ChunkEnd | (nchunks == 1 ? kB3Root : 0u);
        b3_compress(cv, m, nchunks == 1 ? 0ull : c, clen == 0 ? 0u : bl, flags, out);
#pragma unroll
        for (int i = 0; i < 8; ++i) cv[i] = out[i];
    }
    uint32_t* dst = nchunks == 1 ? jb.out8 : jb.scratch + c * 8;
#pragma unroll
    for (int i = 0; i < 8; ++i) dst[i] = cv[i];
}

// Pairwise tree merge, one CTA per job (a lone last node is carried up).
__global__ void __launch_bounds__(1024) hash_tree_jobs_kernel(JobList<HashJob> J) {
    const HashJob jb = J.j[blockIdx.x];
    uint64_t n = jb.len == 0 ? 1 : (jb.len + kB3ChunkLen - 1) / kB3ChunkLen;
    if (n == 1) return;
    const uint32_t iv[8] = {DM_B3_IV0, DM_B3_IV1, DM_B3_IV2, DM_B3_IV3, DM_B3_IV4, DM_B3_IV5, DM_B3_IV6, DM_B3_IV7};
    uint32_t* src = jb.scratch;
    uint32_t* dst = jb.scratch + 8 * n;
    while (n > 1) {
        const uint64_t pairs = n / 2;
        const bool root = (n == 2);
        for (uint64_t j = threadIdx.x; j < pairs; j += blockDim.x) {
            uint32_t m[16], out[16];
#pragma unroll
            for (int i = 0; i < 16; ++i) m[i] = src[2 * j * 8 + i];
            b3_compress(iv, m, 0, 64, kB3Parent | (root ? kB3Root : 0u), out);
            uint32_t* d = root ? jb.out8 : dst + j * 8;
#pragma unroll
            for (int i = 0; i < 8; ++i) d[i] = out[i];
        }
        if ((n & 1) && threadIdx.x == 0)
            for (int i = 0; i < 8; ++i) dst[pairs * 8 + i] = src[(n - 1) * 8 + i];
        __syncthreads();
        n = pairs + (n & 1);
        uint32_t* t = src;
        src = dst;
        dst = t;
    }
}

// ---------------------------------------------------------------- launch helpers
template <class J>
uint32_t assign_ctas(J* jobs, int n, JobList<J>& L, uint64_t (*ctas_of)(const J&)) {
    uint64_t total = 0;
    L.n = n;
    for (int i = 0; i < n; ++i) {
        jobs[i].cta0 = (uint32_t)total;
        L.j[i] = jobs[i];
        total += ctas_of(jobs[i]);
    }
    return (uint32_t)total;
}

template <int L>
cudaError_t ntt_launch_L(const DeviceTables& T, JobList<NttJob>& JL, NttJob* jobs, int n, cudaStream_t st) {
    if constexpr (L < 4) {
        const uint32_t ctas = assign_ctas<NttJob>(jobs, n, JL, [](const NttJob& j) -> uint64_t {
            return (j.npolys * 8ull + 127) / 128;
        });
        if (!ctas) return cudaSuccess;
        ntt_fwd_small_kernel<L><<<ctas, 128, 0, st>>>(JL, T.pc, T.zeta, T.zetap);
    } else {
        using S = NttShape<L>;
        const uint32_t ctas = assign_ctas<NttJob>(jobs, n, JL, [](const NttJob& j) -> uint64_t {
            return ((j.npolys + S::P - 1) / S::P) * S::SPLIT;
        });
        if (!ctas) return cudaSuccess;
        ntt_fwd_jobs_kernel<L><<<ctas, S::THREADS, S::SMEM, st>>>(JL, T.pc, T.zeta, T.zetap);
    }
    return cudaGetLastError();
}

template <int L>
cudaError_t finish_launch_L(const DeviceTables& T, JobList<FinishJobX>& JL, int n, const FinishConsts& plain,
                            const FinishConsts& split, cudaStream_t st) {
    if constexpr (L < 4) {
        finish_small_kernel<L><<<dim3(1, n), 64, 0, st>>>(JL, T.pc, T.cc, plain, split, T.zeta, T.zetap, T.zinv,
                                                           T.zinvp);
    } else {
        using S = FinShape<L>;
        finish_jobs_kernel<L><<<dim3(kRank, n), S::THREADS, S::SMEM, st>>>(JL, T.pc, T.cc, plain, split, T.zeta,
                                                                           T.zetap, T.zinv, T.zinvp);
    }
    return cudaGetLastError();
}

template <int L>
cudaError_t set_smem_attrs() {
    cudaError_t e = cudaSuccess;
    if constexpr (L >= 4) {
        e = cudaFuncSetAttribute((const void*)ntt_fwd_jobs_kernel<L>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)NttShape<L>::SMEM);
        if (e == cudaSuccess && L <= 11)
            e = cudaFuncSetAttribute((const void*)finish_jobs_kernel<(L <= 11 ? L : 11)>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FinShape<(L <= 11 ? L : 11)>::SMEM);
    }
    if (e != cudaSuccess) return e;
    if constexpr (L < kLogMaxProverRing) return set_smem_attrs<L + 1>();
    return cudaSuccess;
}

}  // namespace

// Per device: twiddle-product tables and the shared-memory limits of the templated kernels.
cudaError_t upload_tables_ext(DeviceTables* t) {
    cudaError_t ea = set_smem_attrs<0>();
    if (ea != cudaSuccess) return ea;
    const HostTables& H = host_tables();
    const size_t bytes = sizeof(uint32_t) * H.zetap.size();
    uint32_t *a = nullptr, *b = nullptr;
    cudaError_t e = cudaMalloc(&a, bytes);
    if (e != cudaSuccess) return e;
    if ((e = cudaMalloc(&b, bytes)) != cudaSuccess) {
        cudaFree(a);
        return e;
    }
    e = cudaMemcpy(a, H.zetap.data(), bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b, H.zinvp.data(), bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(a);
        cudaFree(b);
        return e;
    }
    t->zetap = a;
    t->zinvp = b;
    return cudaSuccess;
}

cudaError_t launch_ntt_jobs(const DeviceTables& T, NttJob* jobs, int n, uint32_t L, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs || L > (uint32_t)kLogMaxProverRing) return cudaErrorInvalidValue;
    JobList<NttJob> JL;
    switch (L) {
        case 0: return ntt_launch_L<0>(T, JL, jobs, n, st);
        case 1: return ntt_launch_L<1>(T, JL, jobs, n, st);
        case 2: return ntt_launch_L<2>(T, JL, jobs, n, st);
        case 3: return ntt_launch_L<3>(T, JL, jobs, n, st);
        case 4: return ntt_launch_L<4>(T, JL, jobs, n, st);
        case 5: return ntt_launch_L<5>(T, JL, jobs, n, st);
        case 6: return ntt_launch_L<6>(T, JL, jobs, n, st);
        case 7: return ntt_launch_L<7>(T, JL, jobs, n, st);
        case 8: return ntt_launch_L<8>(T, JL, jobs, n, st);
        case 9: return ntt_launch_L<9>(T, JL, jobs, n, st);
        case 10: return ntt_launch_L<10>(T, JL, jobs, n, st);
        case 11: return ntt_launch_L<11>(T, JL, jobs, n, st);
        case 12: return ntt_launch_L<12>(T, JL, jobs, n, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_mac_triple_jobs(const DeviceTables& T, MacJobX* jobs, int n, uint32_t L, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs) return cudaErrorInvalidValue;
    JobList<MacJobX> JL;
    const uint32_t slots = 1u << L;
    uint64_t total = 0;
    JL.n = n;
    for (int i = 0; i < n; ++i) {
        jobs[i].cta0 = (uint32_t)total;
        JL.j[i] = jobs[i];
        total += (uint64_t)((slots + kMacThreads - 1) / kMacThreads) * 64 * jobs[i].parts;
    }
    const unsigned bx = slots < (uint32_t)kMacThreads ? slots : kMacThreads;
    mac_triple_jobs_kernel<<<(unsigned)total, bx, 0, st>>>(JL, L, T.pc);
    return cudaGetLastError();
}

cudaError_t launch_mac_jobs(const DeviceTables& T, MacJobX* jobs, int n, uint32_t L, bool split, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs || (split && L == 0)) return cudaErrorInvalidValue;
    JobList<MacJobX> JL;
    const uint32_t slots = split ? (1u << (L - 1)) : (1u << L);
    uint64_t total = 0;
    JL.n = n;
    for (int i = 0; i < n; ++i) {
        jobs[i].cta0 = (uint32_t)total;
        JL.j[i] = jobs[i];
        total += (uint64_t)((slots + kMacThreads - 1) / kMacThreads) * 64 * jobs[i].parts;
    }
    const unsigned bx = slots < (uint32_t)kMacThreads ? slots : kMacThreads;
    if (split)
        mac_split_jobs_kernel<<<(unsigned)total, bx, 0, st>>>(JL, L, T.pc);
    else
        mac_jobs_kernel<<<(unsigned)total, bx, 0, st>>>(JL, L, T.pc);
    return cudaGetLastError();
}

cudaError_t launch_finish_jobs(const DeviceTables& T, FinishJobX* jobs, int n, uint32_t L, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs || L > 11) return cudaErrorInvalidValue;
    JobList<FinishJobX> JL;
    JL.n = n;
    for (int i = 0; i < n; ++i) JL.j[i] = jobs[i];
    FinishConsts plain, split;
    for (int i = 0; i < kPrimes; ++i) {
        plain.f[i] = T.ninv_r2[i][L];
        plain.fp[i] = plain.f[i] * T.pc.pinv[i];
        split.f[i] = T.ninv4_r2[i][L];
        split.fp[i] = split.f[i] * T.pc.pinv[i];
    }
    switch (L) {
        case 0: return finish_launch_L<0>(T, JL, n, plain, split, st);
        case 1: return finish_launch_L<1>(T, JL, n, plain, split, st);
        case 2: return finish_launch_L<2>(T, JL, n, plain, split, st);
        case 3: return finish_launch_L<3>(T, JL, n, plain, split, st);
        case 4: return finish_launch_L<4>(T, JL, n, plain, split, st);
        case 5: return finish_launch_L<5>(T, JL, n, plain, split, st);
        case 6: return finish_launch_L<6>(T, JL, n, plain, split, st);
        case 7: return finish_launch_L<7>(T, JL, n, plain, split, st);
        case 8: return finish_launch_L<8>(T, JL, n, plain, split, st);
        case 9: return finish_launch_L<9>(T, JL, n, plain, split, st);
        case 10: return finish_launch_L<10>(T, JL, n, plain, split, st);
        case 11: return finish_launch_L<11>(T, JL, n, plain, split, st);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_fold_jobs(FoldJob* jobs, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs) return cudaErrorInvalidValue;
    JobList<FoldJob> JL;
    const uint32_t ctas = assign_ctas<FoldJob>(jobs, n, JL, [](const FoldJob& j) -> uint64_t {
        return (j.n + kFoldThreads * kFoldItems - 1) / (kFoldThreads * kFoldItems);
    });
    if (!ctas) return cudaSuccess;
    fold_jobs_kernel<<<ctas, kFoldThreads, 0, st>>>(JL);
    return cudaGetLastError();
}

cudaError_t launch_gen_jobs(GenJob* jobs, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs) return cudaErrorInvalidValue;
    JobList<GenJob> JL;
    const uint32_t ctas = assign_ctas<GenJob>(jobs, n, JL, [](const GenJob& j) -> uint64_t {
        return (j.total + kGenThreads * kGenItems - 1) / (kGenThreads * kGenItems);
    });
    if (!ctas) return cudaSuccess;
    gen_jobs_kernel<<<ctas, kGenThreads, 0, st>>>(JL);
    return cudaGetLastError();
}

cudaError_t launch_unpack_jobs(UnpackJob* jobs, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs) return cudaErrorInvalidValue;
    JobList<UnpackJob> JL;
    const uint32_t ctas = assign_ctas<UnpackJob>(jobs, n, JL,
                                                 [](const UnpackJob& j) -> uint64_t { return (j.total + 255) / 256; });
    if (!ctas) return cudaSuccess;
    unpack_jobs_kernel<<<ctas, 256, 0, st>>>(JL);
    return cudaGetLastError();
}

cudaError_t launch_hash_jobs(HashJob* jobs, int n, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs) return cudaErrorInvalidValue;
    JobList<HashJob> JL;
    const uint32_t ctas = assign_ctas<HashJob>(jobs, n, JL, [](const HashJob& j) -> uint64_t {
        const uint64_t c = j.len == 0 ? 1 : (j.len + kB3ChunkLen - 1) / kB3ChunkLen;
        return (c + 127) / 128;
    });
    hash_chunk_jobs_kernel<<<ctas, 128, 0, st>>>(JL);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    hash_tree_jobs_kernel<<<n, 1024, 0, st>>>(JL);
    return cudaGetLastError();
}

}  // namespace dm
