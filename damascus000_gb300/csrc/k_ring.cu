// Ring arithmetic of the commitment and fold stages on the nine NTT primes:
// forward negacyclic transforms, column multiply-accumulates in the NTT domain,
// and the finish (sum of column partials, inverse transform, Garner CRT into
// Z_q, optional compare).  The product of two rings in R_q is exact: every
// commitment sum |X| < N n q^2 < P / 2 is recovered from its residues
// (src/algebra/ntt.rs:112-224, 372-427 computes the same integers per product).
//
// Forward transform: Cooley-Tukey with the negacyclic twist merged into the
// twiddles (zeta[k] = psi^brv(k), psi a primitive 2n-th root), natural order in,
// bit-reversed evaluation order out: slot j holds a(psi^(2 brv(j) + 1)).  Slots
// 2i and 2i+1 are the evaluations at +w_i and -w_i with w_i = zeta[n/2 + i], so
// the even/odd halves of a polynomial are one butterfly layer away.  Inverse:
// Gentleman-Sande with zeta^-1 and a final n^-1.
//
// Block shape of the transforms: rows of 2^L residues (one polynomial under one
// prime), 2^(L-4) threads per polynomial holding 16 residues of each row in
// registers.  A forward-transform thread carries three primes (three blocks per
// polynomial: every coefficient is read once per three residues); an inverse
// thread one.  Small rings put several polynomials in a block (64 threads up to
// L = 10, 2^(L-4) above).
#include <cuda_runtime.h>

#include "dm_jobkit.cuh"
#include "dm_ntt.cuh"
#include "dm_tables.h"

namespace dm {

namespace {

using namespace jobkit;

constexpr int kGroups = kPrimes / kPrimesPerThread;  // forward-transform blocks per polynomial group
constexpr int kRows = kRank * kPrimes;               // MAC rows per job (coordinate, prime)

#ifndef DM_ROW_GROUP_THREADS
#define DM_ROW_GROUP_THREADS 64  // threads per block for small rings (32 or 64)
#endif
static_assert(DM_ROW_GROUP_THREADS == 32 || DM_ROW_GROUP_THREADS == 64, "row barriers assume this");
#ifndef DM_RESIDENT_WARPS
#define DM_RESIDENT_WARPS 32
#endif
#ifndef DM_FWD_RESIDENT_WARPS
#define DM_FWD_RESIDENT_WARPS (DM_RESIDENT_WARPS / kPrimesPerThread > 16 ? DM_RESIDENT_WARPS / kPrimesPerThread : 16)
#endif

// Block shape of the inverse transforms: one row (polynomial under one prime)
// of 2^(L-4) threads, several rows per block for small rings.
template <int L>
struct RowShape {
    static constexpr int T = 1 << (L - 4);                   // threads per row
    static constexpr int P = T >= DM_ROW_GROUP_THREADS ? 1 : DM_ROW_GROUP_THREADS / T;  // rows per block
    static constexpr int ROWS = P;
    static constexpr int THREADS = ROWS * T;
    static constexpr int PASSES = (L + 3) / 4;
    static constexpr size_t SMEM = PASSES > 1 ? (size_t)ROWS * (1u << L) * sizeof(uint32_t) : 0;
};

// Block shape of the forward transforms: P polynomials, each held by 2^(L-4)
// threads with kPrimesPerThread residue rows per thread; shared memory holds
// kPrimesPerThread x P rows, prime-major, so each prime's rows sit together as
// in a one-prime block.
// LE: the pass radix, 2^LE residues per thread (4, or 5 for the radix-32
// alternative the kTuneNttRadix knob selects).
template <int L, int G = DM_ROW_GROUP_THREADS, int LE = kNttLogE>
struct FwdShape {
    static_assert(G == 32 || G == 64, "row groups of 32 or 64 threads");
    static_assert(LE == 4 || LE == 5, "radix-16 or radix-32 passes");
    static constexpr int T = 1 << (L - LE);
    static constexpr int P = T >= G ? 1 : G / T;
    static constexpr int THREADS = P * T;
    static constexpr int PASSES = (L + LE - 1) / LE;
    static constexpr size_t SMEM = PASSES > 1 ? (size_t)kPrimesPerThread * P * (1u << L) * sizeof(uint32_t) : 0;
    // resident blocks per SM the register budget is sized for (32 warps per SM
    // with one prime per thread: measured faster than 48 or 64; the registers
    // hold loads in flight).  Radix-32 passes hold twice the residues and
    // twiddles per thread: 16 warps.
    static constexpr int WARPS = LE == kNttLogE ? DM_FWD_RESIDENT_WARPS : 16;
    static constexpr int MIN_BLOCKS = (WARPS * 32) / THREADS > 0 ? (WARPS * 32) / THREADS : 1;
};

// Exchange barrier of one row group: a group of 2^(L-4) consecutive threads that
// fits one warp needs only a warp barrier; larger groups are the whole block.
// Every thread of a group, active or not, runs the same passes and so the same
// barriers.
template <int L, int LE = kNttLogE>
DM_D void row_sync() {
    if constexpr ((1 << (L - LE)) <= 32) {
        __syncwarp();
    } else {
        static_assert(FwdShape<L, 64, LE>::P == 1 && (LE != kNttLogE || RowShape<L>::P == 1),
                      "groups above a warp fill their block");
        __syncthreads();
    }
}

// ================================================================ forward NTT

template <int L, int G, int LE = kNttLogE>
__global__ void __launch_bounds__(FwdShape<L, G, LE>::THREADS, FwdShape<L, G, LE>::MIN_BLOCKS)
    ntt_fwd_kernel(JobList<NttJob> J, PrimeConsts pc, const Tw* __restrict__ fwd, const Tw* __restrict__ fwd_last) {
    using S = FwdShape<L, G, LE>;
    constexpr int K = kPrimesPerThread;
    constexpr int E = 1 << LE;
    extern __shared__ __align__(16) uint32_t sm[];
    const NttJob jb = J.j[find_job(J)];
    const uint32_t lcta = blockIdx.x - jb.cta0;
    const uint32_t grp = lcta / kGroups, pi0 = (lcta % kGroups) * K;
    const uint32_t prow = threadIdx.x / S::T;  // polynomial within the block
    const uint32_t t = threadIdx.x % S::T;
    const uint64_t poly = (uint64_t)grp * S::P + prow;
    const bool active = poly < jb.npolys;
    uint32_t a[K][E];
    if (active) {
        const uint4* src = jb.src + (poly << L);
#pragma unroll
        for (int r = 0; r < E; ++r) {
            const fq x = ldq(src, ntt_place_e<LE>(L, 0, t, r));
#pragma unroll
            for (int k = 0; k < K; ++k) a[k][r] = residue_fwd(x, pc, pi0 + k);
        }
    } else {
#pragma unroll
        for (int k = 0; k < K; ++k)
#pragma unroll
            for (int r = 0; r < E; ++r) a[k][r] = 0;
    }
#pragma unroll
    for (int pass = 0; pass < S::PASSES; ++pass) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            if constexpr (LE == kNttLogE)
                ntt_fwd_pass(a[k], L, pass, t, fwd + (pi0 + k) * kMaxRing,
                             fwd_last + (pi0 + k) * kLastSpan + (1u << L) - 16u, pc.p[pi0 + k]);
            else
                ntt_fwd_pass_e<LE>(a[k], L, pass, t, fwd + (pi0 + k) * kMaxRing, pc.p[pi0 + k]);
        }
        if (pass + 1 < S::PASSES) {
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const uint32_t ws = ntt_swz_base_e<LE>((uint32_t)(k * S::P + prow) << L, L, pass, t);
#pragma unroll
                for (int r = 0; r < E; ++r) sm[ws ^ ntt_swz_reg_e<LE>(L, pass, r)] = a[k][r];
            }
            row_sync<L, LE>();
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const uint32_t rs = ntt_swz_base_e<LE>((uint32_t)(k * S::P + prow) << L, L, pass + 1, t);
#pragma unroll
                for (int r = 0; r < E; ++r) a[k][r] = sm[rs ^ ntt_swz_reg_e<LE>(L, pass + 1, r)];
            }
            row_sync<L, LE>();
        }
    }
    if (active) {
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const uint32_t pi = pi0 + k, p = pc.p[pi], one_s = pc.one_s[pi];
#pragma unroll
            for (int r = 0; r < E; ++r) a[k][r] = ntt_fwd_final(a[k][r], one_s, p);
            // the last pass holds slots E t .. E t + E - 1
            uint4* dst = reinterpret_cast<uint4*>(jb.dst + ((poly * kPrimes + pi) << L) + t * E);
#pragma unroll
            for (int q = 0; q < E / 4; ++q)
                dst[q] = make_uint4(a[k][4 * q], a[k][4 * q + 1], a[k][4 * q + 2], a[k][4 * q + 3]);
        }
    }
}

// Rings smaller than 16: one thread per (polynomial, prime), all in registers.
template <int L>
__global__ void __launch_bounds__(128) ntt_fwd_small_kernel(JobList<NttJob> J, PrimeConsts pc,
                                                            const Tw* __restrict__ fwd) {
    constexpr int s = 1 << L;
    const NttJob jb = J.j[find_job(J)];
    const uint64_t item = (uint64_t)(blockIdx.x - jb.cta0) * blockDim.x + threadIdx.x;
    const uint64_t poly = item / kPrimes;
    const uint32_t pi = (uint32_t)(item % kPrimes);
    if (poly >= jb.npolys) return;
    const uint32_t p = pc.p[pi];
    uint32_t a[s];
#pragma unroll
    for (int c = 0; c < s; ++c) a[c] = residue_fwd(ldq(jb.src + (poly << L), c), pc, pi);
    ntt_fwd_small<L>(a, fwd + pi * kMaxRing, p);
#pragma unroll
    for (int c = 0; c < s; ++c) jb.dst[((poly * kPrimes + pi) << L) + c] = ntt_fwd_final(a[c], pc.one_s[pi], p);
}

// ================================================================ MAC
// Residues are < p < 2^28, so a product fits 56 bits and 16 of them fit a
// 64-bit word with room to spare; block sums go into a 96-bit accumulator (64-bit low word + carry
// count) reduced once per output.
constexpr int kMacThreads = 128;

DM_D uint32_t slot_block_count(uint32_t s) { return (s + kMacThreads - 1) / kMacThreads; }
DM_D void acc96(uint64_t& lo, uint32_t& hi, uint64_t v) {
    lo += v;
    hi += lo < v ? 1u : 0u;
}
DM_D uint64_t mul64(uint32_t a, uint32_t b) { return (uint64_t)a * b; }

// grid: per job, nblk * 72 * parts blocks; block -> (part, row, slot block).
__global__ void __launch_bounds__(kMacThreads) mac_jobs_kernel(JobList<MacJobX> J, PrimeConsts pc) {
    const MacJobX jb = J.j[find_job(J)];
    const uint32_t L = jb.L;
    const uint32_t s = 1u << L;
    const uint32_t nblk = slot_block_count(s);
    uint32_t c = blockIdx.x - jb.cta0;
    const uint32_t blk = c % nblk;
    c /= nblk;
    const uint32_t kp = c % kRows;
    const uint32_t part = c / kRows;
    const uint32_t slot = blk * kMacThreads + threadIdx.x;
    if (slot >= s) return;
    const uint32_t k = kp / kPrimes, pi = kp % kPrimes;
    const uint32_t i0 = (uint32_t)((uint64_t)jb.count * part / jb.parts);
    const uint32_t i1 = (uint32_t)((uint64_t)jb.count * (part + 1) / jb.parts);
    const uint64_t gstride = (uint64_t)kRank * kPrimes << L;  // one generator vector
    const uint64_t mstride = (uint64_t)kPrimes << L;
    const uint32_t* g = jb.G + ((((uint64_t)jb.g_base * kRank + k) * kPrimes + pi) << L) + slot;
    const uint32_t* m = jb.M + (((uint64_t)jb.m_base * kPrimes + pi) << L) + slot;
    uint64_t lo = 0;
    uint32_t hi = 0;
    uint32_t i = i0;
    for (; i + 8 <= i1; i += 8) {
        uint64_t b0 = 0, b1 = 0;
#pragma unroll
        for (int u = 0; u < 8; u += 2) {
            b0 += mul64(__ldg(g + (i + u) * gstride), __ldg(m + (i + u) * mstride));
            b1 += mul64(__ldg(g + (i + u + 1) * gstride), __ldg(m + (i + u + 1) * mstride));
        }
        acc96(lo, hi, b0);
        acc96(lo, hi, b1);
    }
    uint64_t b = 0;
    for (; i < i1; ++i) b += mul64(__ldg(g + i * gstride), __ldg(m + i * mstride));
    acc96(lo, hi, b);
    jb.out0[(((uint64_t)part * kRows + kp) << L) + slot] = red96(hi, lo, pc, pi);
}

// Triple MAC over column pairs (i, i + h): one read of every generator column
// gives the full sum (out0), L = sum G[i+h] M[i] (out1) and R = sum G[i] M[i+h]
// (out2).  h = count, or h = pair when the witness columns from h on are known
// zero: then i runs over the count < h leading columns only, the witness is read
// at i alone and R is zero.  Thread per slot pair (8-byte loads), L >= 1, and KC
// commitment coordinates of one prime: each column's witness slot pairs are
// loaded once for the KC generator rows.
template <int KC, bool PAIR>
DM_D void triple_rows(const MacJobX& jb, uint32_t kg, uint32_t pi, uint32_t part, uint32_t i2, const PrimeConsts& pc) {
    const uint32_t L = jb.L;
    const uint32_t h = PAIR ? jb.pair : jb.count;
    const uint32_t i0 = (uint32_t)((uint64_t)jb.count * part / jb.parts);
    const uint32_t i1 = (uint32_t)((uint64_t)jb.count * (part + 1) / jb.parts);
    const uint64_t gstride = (uint64_t)kRank * kPrimes << L;
    const uint64_t mstride = (uint64_t)kPrimes << L;
    const uint64_t kstride = (uint64_t)kPrimes << L;  // the next coordinate's row, same prime
    const uint32_t* g = jb.G + ((((uint64_t)kg * KC) * kPrimes + pi) << L) + 2 * i2;
    const uint32_t* m = jb.M + (((uint64_t)pi) << L) + 2 * i2;
    const uint64_t gh = (uint64_t)h * gstride, mh = (uint64_t)h * mstride;
    constexpr int NS = PAIR ? 4 : 6;  // sums per coordinate: (full, L[, R]) x (even, odd slot)
    uint64_t lo[KC][NS];
    uint32_t hi[KC][NS];
#pragma unroll
    for (int j = 0; j < KC; ++j)
#pragma unroll
        for (int q = 0; q < NS; ++q) lo[j][q] = 0, hi[j][q] = 0;
    // products below 2^56: a block sum of up to 256 of them fits 64 bits; a block of
    // 16 columns sums 16 (pair) or 32 (full: two products per sum)
#ifndef DM_TRIPLE_FULL_BLOCK
#define DM_TRIPLE_FULL_BLOCK 8
#endif
#ifndef DM_TRIPLE_UNROLL1
#define DM_TRIPLE_UNROLL1 4
#endif
    constexpr uint32_t kBlock = PAIR ? 16 : DM_TRIPLE_FULL_BLOCK;
    static_assert(DM_TRIPLE_FULL_BLOCK <= 64, "block sums of 2 x 64 products below 2^56 fit 64 bits");
    constexpr int kUnroll = KC >= 4 ? 2 : (KC == 2 ? 2 : DM_TRIPLE_UNROLL1);
    uint32_t i = i0;
    while (i < i1) {
        const uint32_t e = i + kBlock < i1 ? i + kBlock : i1;
        uint64_t b[KC][NS];
#pragma unroll
        for (int j = 0; j < KC; ++j)
#pragma unroll
            for (int q = 0; q < NS; ++q) b[j][q] = 0;
#pragma unroll kUnroll
        for (; i < e; ++i) {
            const uint2 ml = __ldg(reinterpret_cast<const uint2*>(m + i * mstride));
            uint2 mr = make_uint2(0u, 0u);
            if (!PAIR) mr = __ldg(reinterpret_cast<const uint2*>(m + i * mstride + mh));
#pragma unroll
            for (int j = 0; j < KC; ++j) {
                const uint2 gl = __ldg(reinterpret_cast<const uint2*>(g + i * gstride + j * kstride));
                const uint2 gr = __ldg(reinterpret_cast<const uint2*>(g + i * gstride + j * kstride + gh));
                if (PAIR) {
                    b[j][0] += mul64(gl.x, ml.x);
                    b[j][1] += mul64(gl.y, ml.y);
                    b[j][2] += mul64(gr.x, ml.x);
                    b[j][3] += mul64(gr.y, ml.y);
                } else {
                    b[j][0] += mul64(gl.x, ml.x) + mul64(gr.x, mr.x);
                    b[j][1] += mul64(gl.y, ml.y) + mul64(gr.y, mr.y);
                    b[j][2] += mul64(gr.x, ml.x);
                    b[j][3] += mul64(gr.y, ml.y);
                    b[j][4] += mul64(gl.x, mr.x);
                    b[j][5] += mul64(gl.y, mr.y);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < KC; ++j)
#pragma unroll
            for (int q = 0; q < NS; ++q) acc96(lo[j][q], hi[j][q], b[j][q]);
    }
#pragma unroll
    for (int j = 0; j < KC; ++j) {
        const uint64_t row = (uint64_t)part * kRows + (kg * KC + j) * kPrimes + pi;
        const uint64_t o = (row << L) + 2 * i2;
        *reinterpret_cast<uint2*>(jb.out0 + o) =
            make_uint2(red96(hi[j][0], lo[j][0], pc, pi), red96(hi[j][1], lo[j][1], pc, pi));
        *reinterpret_cast<uint2*>(jb.out1 + o) =
            make_uint2(red96(hi[j][2], lo[j][2], pc, pi), red96(hi[j][3], lo[j][3], pc, pi));
        *reinterpret_cast<uint2*>(jb.out2 + o) =
            PAIR ? make_uint2(0u, 0u)
                 : make_uint2(red96(hi[j][NS - 2], lo[j][NS - 2], pc, pi), red96(hi[j][NS - 1], lo[j][NS - 1], pc, pi));
    }
}

// grid: per job, nblk * (72 / KC) * parts blocks; every job of a launch has kc == KC.
template <int KC>
__global__ void __launch_bounds__(kMacThreads) mac_triple_jobs_kernel(JobList<MacJobX> J, PrimeConsts pc) {
    const MacJobX jb = J.j[find_job(J)];
    const uint32_t sp = 1u << (jb.L - 1);
    const uint32_t nblk = slot_block_count(sp);
    constexpr uint32_t rows = kRows / KC;
    uint32_t c = blockIdx.x - jb.cta0;
    const uint32_t blk = c % nblk;
    c /= nblk;
    const uint32_t kp = c % rows;
    const uint32_t part = c / rows;
    const uint32_t i2 = blk * kMacThreads + threadIdx.x;
    if (i2 >= sp) return;
    if (jb.pair)
        triple_rows<KC, true>(jb, kp / kPrimes, kp % kPrimes, part, i2, pc);
    else
        triple_rows<KC, false>(jb, kp / kPrimes, kp % kPrimes, part, i2, pc);
}

// Split MAC: thread per slot pair (2 i2, 2 i2 + 1) of ring 2^L (L >= 1) and KC
// commitment coordinates of one prime: the recompute check over all slots and
// the even/odd cross terms (g(w) - g(-w)) (m(w) + m(-w)) and
// (g(w) + g(-w)) (m(w) - m(-w)) at 2^(L-1).  Each column's witness slot pair is
// loaded once for the KC generator rows (and its sum and difference formed once).
template <int KC>
DM_D void split_rows(const MacJobX& jb, uint32_t kg, uint32_t pi, uint32_t part, uint32_t i2, const PrimeConsts& pc) {
    const uint32_t L = jb.L;
    const uint32_t i0 = (uint32_t)((uint64_t)jb.count * part / jb.parts);
    const uint32_t i1 = (uint32_t)((uint64_t)jb.count * (part + 1) / jb.parts);
    const uint32_t p = pc.p[pi];
    const uint64_t gstride = (uint64_t)kRank * kPrimes << L;
    const uint64_t mstride = (uint64_t)kPrimes << L;
    const uint64_t kstride = (uint64_t)kPrimes << L;  // the next coordinate's row, same prime
    const uint32_t* g = jb.G + ((((uint64_t)jb.g_base * kRank + kg * KC) * kPrimes + pi) << L) + 2 * i2;
    const uint32_t* m = jb.M + (((uint64_t)jb.m_base * kPrimes + pi) << L) + 2 * i2;
    uint64_t l0[KC], l1[KC], ll[KC], lr[KC];
    uint32_t h0[KC], h1[KC], hl[KC], hr[KC];
#pragma unroll
    for (int j = 0; j < KC; ++j) l0[j] = l1[j] = ll[j] = lr[j] = 0, h0[j] = h1[j] = hl[j] = hr[j] = 0;
    // columns unrolled: measured best 8, 4, 2 and 4 for 1, 2, 4 and 8 coordinates per
    // thread (eight coordinates: 243 registers, two blocks per SM, and four columns
    // of loads in flight time 0.228 ms at 2^11 over 2048 columns against 0.285
    // with two)
    constexpr int kUnroll = KC == 8 ? 4 : (KC == 4 ? 2 : 8 / KC);
    uint32_t i = i0;
    while (i < i1) {
        const uint32_t e = i + 16 < i1 ? i + 16 : i1;
        uint64_t b0[KC], b1[KC], bl[KC], br[KC];
#pragma unroll
        for (int j = 0; j < KC; ++j) b0[j] = b1[j] = bl[j] = br[j] = 0;
#pragma unroll kUnroll
        for (; i < e; ++i) {
            const uint2 mv = __ldg(reinterpret_cast<const uint2*>(m + i * mstride));
            // sums and differences below 2p: products below 4p^2 < 2^58, 16 of them fit
            const uint32_t msum = mv.x + mv.y, mdif = mv.x + p - mv.y;
#pragma unroll
            for (int j = 0; j < KC; ++j) {
                const uint2 gv = __ldg(reinterpret_cast<const uint2*>(g + i * gstride + j * kstride));
                b0[j] += mul64(gv.x, mv.x);
                b1[j] += mul64(gv.y, mv.y);
                bl[j] += mul64(gv.x + p - gv.y, msum);
                br[j] += mul64(gv.x + gv.y, mdif);
            }
        }
#pragma unroll
        for (int j = 0; j < KC; ++j) {
            acc96(l0[j], h0[j], b0[j]);
            acc96(l1[j], h1[j], b1[j]);
            acc96(ll[j], hl[j], bl[j]);
            acc96(lr[j], hr[j], br[j]);
        }
    }
#pragma unroll
    for (int j = 0; j < KC; ++j) {
        const uint64_t row = (uint64_t)part * kRows + (kg * KC + j) * kPrimes + pi;
        *reinterpret_cast<uint2*>(jb.out0 + (row << L) + 2 * i2) =
            make_uint2(red96(h0[j], l0[j], pc, pi), red96(h1[j], l1[j], pc, pi));
        jb.out1[(row << (L - 1)) + i2] = red96(hl[j], ll[j], pc, pi);
        jb.out2[(row << (L - 1)) + i2] = red96(hr[j], lr[j], pc, pi);
    }
}

// grid: per job, nblk * (72 / KC) * parts blocks; block -> (part, coordinate group x prime, slot block).
// Every job of a launch has kc == KC (the launcher groups them).
template <int KC>
__global__ void __launch_bounds__(kMacThreads) mac_split_jobs_kernel(JobList<MacJobX> J, PrimeConsts pc) {
    const MacJobX jb = J.j[find_job(J)];
    const uint32_t hs = 1u << (jb.L - 1);
    const uint32_t nblk = slot_block_count(hs);
    constexpr uint32_t rows = kRows / KC;
    uint32_t c = blockIdx.x - jb.cta0;
    const uint32_t blk = c % nblk;
    c /= nblk;
    const uint32_t kp = c % rows;
    const uint32_t part = c / rows;
    const uint32_t i2 = blk * kMacThreads + threadIdx.x;
    if (i2 >= hs) return;
    split_rows<KC>(jb, kp / kPrimes, kp % kPrimes, part, i2, pc);
}

// ================================================================ finish
struct FinishConsts {
    uint32_t f[kPrimes], fs[kPrimes];  // final inverse-transform scale and its Shoup constant
};

DM_D uint32_t twist(uint32_t x, uint32_t mode, uint32_t idx, const Tw* fwd, const Tw* inv, uint32_t p) {
    if (mode == kFinishSplitL) return shoup_mul(x, fwd[idx], p);
    if (mode == kFinishSplitR) return shoup_mul(x, inv[idx], p);
    return x;
}

// The row part of a finish: the row's input (the sum of its column partials, or
// the slotwise product of two transformed rows), the split twist (w_i or w_i^-1;
// the 1/4 is in the final scale), the inverse transform through the row's
// shared-memory slice at `base` and the final scale.  Leaves the row's residues
// in a (register r of thread t holds coefficient place(L, 0, t, r)).  Every
// thread of a row group runs the same passes and barriers, active or not.
template <int L>
DM_D void finish_row(const FinishJobX& jb, uint32_t row, uint32_t t, uint32_t base, bool active, const PrimeConsts& pc,
                     const FinishConsts& plain, const FinishConsts& split, const Tw* __restrict__ fwd,
                     const Tw* __restrict__ inv, const Tw* __restrict__ inv_last, uint32_t* sm, uint32_t a[kNttE]) {
    constexpr uint32_t s = 1u << L;
    constexpr int PASSES = (L + 3) / 4;
    const uint32_t pi = active ? row % kPrimes : 0;
    const uint32_t p = pc.p[pi];
#pragma unroll
    for (int r = 0; r < kNttE; ++r) a[r] = 0;
    if (active) {
        const uint4* src = reinterpret_cast<const uint4*>(jb.partials + ((uint64_t)row << L) + t * kNttE);
        if (jb.rhs) {
            // slotwise product of two transformed rows, below 4p
            const uint4* sb = reinterpret_cast<const uint4*>(jb.rhs + ((uint64_t)row << L) + t * kNttE);
#pragma unroll
            for (int q4 = 0; q4 < 4; ++q4) {
                const uint4 u = src[q4], v = sb[q4];
                a[4 * q4] = red64_lazy(mul64(u.x, v.x), pc, pi);
                a[4 * q4 + 1] = red64_lazy(mul64(u.y, v.y), pc, pi);
                a[4 * q4 + 2] = red64_lazy(mul64(u.z, v.z), pc, pi);
                a[4 * q4 + 3] = red64_lazy(mul64(u.w, v.w), pc, pi);
            }
        } else {
            // plain 32-bit sums (at most kMaxMacParts residues below 2^28), loads of
            // several parts in flight, one reduction at the end
            const uint64_t pstep = ((uint64_t)jb.rows << L) / 4;  // one part, in uint4
#pragma unroll 4
            for (uint32_t part = 0; part < jb.parts; ++part) {
#pragma unroll
                for (int q4 = 0; q4 < 4; ++q4) {
                    const uint4 v = src[part * pstep + q4];
                    a[4 * q4] += v.x;
                    a[4 * q4 + 1] += v.y;
                    a[4 * q4 + 2] += v.z;
                    a[4 * q4 + 3] += v.w;
                }
            }
        }
        // to [0, 2p): the twist's Shoup product takes any 32-bit value
        const uint32_t one_s = pc.one_s[pi];
#pragma unroll
        for (int r = 0; r < kNttE; ++r)
            a[r] = jb.mode == kFinishPlain ? shoup_one(a[r], one_s, p)
                                           : twist(a[r], jb.mode, pi * kMaxRing + s + t * kNttE + r, fwd, inv, p);
    }
    const Tw* tw = inv + pi * kMaxRing;
    const Tw* twl = inv_last + pi * kLastSpan + (1u << L) - 16u;
#pragma unroll
    for (int pass = PASSES - 1; pass >= 0; --pass) {
        ntt_inv_pass(a, L, pass, t, tw, twl, p);
        if (pass > 0) {
            const uint32_t ws = ntt_swz_base(base, L, pass, t);
#pragma unroll
            for (int r = 0; r < kNttE; ++r) sm[ws ^ ntt_swz_reg(L, pass, r)] = a[r];
            row_sync<L>();
            const uint32_t rs = ntt_swz_base(base, L, pass - 1, t);
#pragma unroll
            for (int r = 0; r < kNttE; ++r) a[r] = sm[rs ^ ntt_swz_reg(L, pass - 1, r)];
            row_sync<L>();
        }
    }
    if (active) {
        const FinishConsts& fc = (jb.mode == kFinishPlain) ? plain : split;
        const uint32_t f = fc.f[pi], fs = fc.fs[pi];
#pragma unroll
        for (int r = 0; r < kNttE; ++r) a[r] = red_below(shoup_mul(a[r], f, fs, p), p);
    }
}

// Block -> ROWS consecutive rows of one job: the row part of the finish, residues
// written over the row's part-0 partials for crt_jobs_kernel.
template <int L>
__global__ void __launch_bounds__(RowShape<L>::THREADS)
    inv_rows_kernel(JobList<FinishJobX> J, PrimeConsts pc, FinishConsts plain, FinishConsts split,
                    const Tw* __restrict__ fwd, const Tw* __restrict__ inv, const Tw* __restrict__ inv_last) {
    using S = RowShape<L>;
    extern __shared__ __align__(16) uint32_t sm[];
    const FinishJobX jb = J.j[find_job(J)];
    const uint32_t brow = threadIdx.x / S::T;
    const uint32_t t = threadIdx.x % S::T;
    const uint32_t row = (blockIdx.x - jb.cta0) * S::ROWS + brow;
    const bool active = row < jb.rows;
    uint32_t a[kNttE];
    finish_row<L>(jb, row, t, brow << L, active, pc, plain, split, fwd, inv, inv_last, sm, a);
    if (active) {
        uint32_t* dst = jb.partials + ((uint64_t)row << L);
#pragma unroll
        for (int r = 0; r < kNttE; ++r) dst[ntt_place(L, 0, t, r)] = a[r];
    }
}

// The whole finish of P polynomials in one block, rings of 2^4 .. 2^10: the
// nine prime rows of each polynomial go through finish_row, stay in shared
// memory, and the same block recombines them by Garner CRT into Z_q (no
// residue round trip through HBM, one launch instead of two).
template <int L>
struct FusedShape {
    static constexpr int T = 1 << (L - 4);
    static constexpr int P = T >= 32 ? 1 : 32 / T;  // polynomials per block
    static constexpr int ROWS = kPrimes * P;
    static constexpr int THREADS = ROWS * T;        // 288 or 576
    static constexpr size_t SMEM = (size_t)ROWS * (1u << L) * sizeof(uint32_t);
};

template <int L>
__global__ void __launch_bounds__(FusedShape<L>::THREADS)
    finish_fused_kernel(JobList<FinishJobX> J, PrimeConsts pc, CrtConsts cc, FinishConsts plain, FinishConsts split,
                        const Tw* __restrict__ fwd, const Tw* __restrict__ inv, const Tw* __restrict__ inv_last) {
    using S = FusedShape<L>;
    constexpr uint32_t s = 1u << L;
    extern __shared__ __align__(16) uint32_t sm[];
    const FinishJobX jb = J.j[find_job(J)];
    const uint32_t brow = threadIdx.x / S::T;
    const uint32_t t = threadIdx.x % S::T;
    const uint32_t poly0 = (blockIdx.x - jb.cta0) * S::P;
    const uint32_t row = poly0 * kPrimes + brow;
    const bool active = row < jb.rows;
    const uint32_t base = brow << L;
    uint32_t a[kNttE];
    finish_row<L>(jb, row, t, base, active, pc, plain, split, fwd, inv, inv_last, sm, a);
    row_sync<L>();  // the row is done reading its exchange slice
#pragma unroll
    for (int r = 0; r < kNttE; ++r) sm[base + ntt_place(L, 0, t, r)] = a[r];
    __syncthreads();
    const uint32_t npolys = jb.rows / kPrimes;
    for (uint32_t idx = threadIdx.x; idx < (uint32_t)S::P * s; idx += S::THREADS) {
        const uint32_t q = idx >> L, j = idx & (s - 1);
        const uint32_t poly = poly0 + q;
        if (poly >= npolys) continue;
        uint32_t r[kPrimes];
#pragma unroll
        for (int i = 0; i < kPrimes; ++i) r[i] = sm[((q * kPrimes + i) << L) + j];
        const fq v = crt_to_fq(r, pc, cc);
        const uint64_t e = ((uint64_t)poly << L) + j;
        stq(jb.out, e, v);
        if (jb.host_out) stq(jb.host_out, e, v);
        if (jb.expect) {
            const uint4 x = jb.expect[e];
            if (x.x != v.w[0] || x.y != v.w[1] || x.z != v.w[2] || x.w != v.w[3]) *jb.flag = 1u;
        }
    }
}

// Rings below 16 coefficients: one thread per row holds the whole row.  The row
// part of the finish (input, twist, inverse, scale) into a[].
template <int L>
DM_D void finish_row_small(const FinishJobX& jb, uint32_t row, const PrimeConsts& pc, const FinishConsts& plain,
                           const FinishConsts& split, const Tw* __restrict__ fwd, const Tw* __restrict__ inv,
                           uint32_t a[1u << L]) {
    constexpr uint32_t s = 1u << L;
    const uint32_t pi = row % kPrimes;
    const uint32_t p = pc.p[pi];
#pragma unroll
    for (uint32_t c = 0; c < s; ++c) a[c] = 0;
    if (jb.rhs) {
#pragma unroll
        for (uint32_t c = 0; c < s; ++c)
            a[c] = red64_lazy(mul64(jb.partials[((uint64_t)row << L) + c], jb.rhs[((uint64_t)row << L) + c]), pc, pi);
    } else {
        for (uint32_t part = 0; part < jb.parts; ++part)  // at most kMaxMacParts residues: no overflow
#pragma unroll
            for (uint32_t c = 0; c < s; ++c) a[c] += jb.partials[(((uint64_t)part * jb.rows + row) << L) + c];
    }
#pragma unroll
    for (uint32_t c = 0; c < s; ++c)
        a[c] = jb.mode == kFinishPlain ? shoup_one(a[c], pc.one_s[pi], p)
                                       : twist(a[c], jb.mode, pi * kMaxRing + s + c, fwd, inv, p);
    ntt_inv_small<L>(a, inv + pi * kMaxRing, p);
    const FinishConsts& fc = (jb.mode == kFinishPlain) ? plain : split;
#pragma unroll
    for (uint32_t c = 0; c < s; ++c) a[c] = red_below(shoup_mul(a[c], fc.f[pi], fc.fs[pi], p), p);
}

// The whole finish of rings below 16 coefficients: P polynomials per block, one
// thread per prime row, the CRT from shared memory in the same block.
constexpr int kFusedSmallPolys = 32;
template <int L>
__global__ void __launch_bounds__(kFusedSmallPolys * kPrimes)
    finish_fused_small_kernel(JobList<FinishJobX> J, PrimeConsts pc, CrtConsts cc, FinishConsts plain,
                              FinishConsts split, const Tw* __restrict__ fwd, const Tw* __restrict__ inv) {
    constexpr uint32_t s = 1u << L;
    __shared__ uint32_t sm[kFusedSmallPolys * kPrimes * s];
    const FinishJobX jb = J.j[find_job(J)];
    const uint32_t poly0 = (blockIdx.x - jb.cta0) * kFusedSmallPolys;
    const uint32_t row = poly0 * kPrimes + threadIdx.x;
    if (row < jb.rows) {
        uint32_t a[s];
        finish_row_small<L>(jb, row, pc, plain, split, fwd, inv, a);
#pragma unroll
        for (uint32_t c = 0; c < s; ++c) sm[threadIdx.x * s + c] = a[c];
    }
    __syncthreads();
    const uint32_t npolys = jb.rows / kPrimes;
    for (uint32_t idx = threadIdx.x; idx < kFusedSmallPolys * s; idx += kFusedSmallPolys * kPrimes) {
        const uint32_t q = idx >> L, j = idx & (s - 1);
        const uint32_t poly = poly0 + q;
        if (poly >= npolys) continue;
        uint32_t r[kPrimes];
#pragma unroll
        for (int i = 0; i < kPrimes; ++i) r[i] = sm[(q * kPrimes + i) * s + j];
        const fq v = crt_to_fq(r, pc, cc);
        const uint64_t e = ((uint64_t)poly << L) + j;
        stq(jb.out, e, v);
        if (jb.host_out) stq(jb.host_out, e, v);
        if (jb.expect) {
            const uint4 x = jb.expect[e];
            if (x.x != v.w[0] || x.y != v.w[1] || x.z != v.w[2] || x.w != v.w[3]) *jb.flag = 1u;
        }
    }
}

// Thread per output coefficient: the nine residues of (poly, slot) -> Z_q.
constexpr int kCrtThreads = 256;
__global__ void __launch_bounds__(kCrtThreads) crt_jobs_kernel(JobList<FinishJobX> J, uint32_t L, PrimeConsts pc,
                                                               CrtConsts cc) {
    const FinishJobX jb = J.j[find_job(J)];
    const uint64_t e = (uint64_t)(blockIdx.x - jb.cta0) * kCrtThreads + threadIdx.x;
    const uint64_t npolys = jb.rows / kPrimes;
    if (e >= (npolys << L)) return;
    const uint64_t poly = e >> L;
    const uint32_t slot = (uint32_t)(e & ((1u << L) - 1));
    uint32_t r[kPrimes];
#pragma unroll
    for (int i = 0; i < kPrimes; ++i) r[i] = jb.partials[((poly * kPrimes + i) << L) + slot];
    const fq v = crt_to_fq(r, pc, cc);
    stq(jb.out, e, v);
    if (jb.host_out) stq(jb.host_out, e, v);
    if (jb.expect) {
        const uint4 x = jb.expect[e];
        if (x.x != v.w[0] || x.y != v.w[1] || x.z != v.w[2] || x.w != v.w[3]) *jb.flag = 1u;
    }
}

// ---------------------------------------------------------------- launch helpers
template <int L, int G, int LE = kNttLogE>
cudaError_t ntt_launch_LG(const DeviceTables& T, JobList<NttJob>& JL, NttJob* jobs, int n, cudaStream_t st) {
    using S = FwdShape<L, G, LE>;
    const uint32_t ctas = assign_ctas<NttJob>(jobs, n, JL, [](const NttJob& j) -> uint64_t {
        return ((uint64_t)(j.npolys + S::P - 1) / S::P) * kGroups;
    });
    if (!ctas) return cudaSuccess;
    ntt_fwd_kernel<L, G, LE><<<ctas, S::THREADS, S::SMEM, st>>>(JL, T.pc, T.fwd, T.fwd_last);
    return cudaGetLastError();
}

template <int L>
cudaError_t ntt_launch_L(const DeviceTables& T, JobList<NttJob>& JL, NttJob* jobs, int n, cudaStream_t st, int group,
                         int elems) {
    if constexpr (L < 4) {
        const uint32_t ctas = assign_ctas<NttJob>(jobs, n, JL, [](const NttJob& j) -> uint64_t {
            return ((uint64_t)j.npolys * kPrimes + 127) / 128;
        });
        if (!ctas) return cudaSuccess;
        ntt_fwd_small_kernel<L><<<ctas, 128, 0, st>>>(JL, T.pc, T.fwd);
    } else {
        if constexpr (L >= 5) {
            if (elems == 32) {
                if constexpr (L < 10)
                    return group == 32 ? ntt_launch_LG<L, 32, 5>(T, JL, jobs, n, st)
                                       : ntt_launch_LG<L, 64, 5>(T, JL, jobs, n, st);
                else
                    return ntt_launch_LG<L, 64, 5>(T, JL, jobs, n, st);
            }
        }
        if constexpr (L < 10)
            return group == 32 ? ntt_launch_LG<L, 32>(T, JL, jobs, n, st) : ntt_launch_LG<L, 64>(T, JL, jobs, n, st);
        else
            return ntt_launch_LG<L, 64>(T, JL, jobs, n, st);
    }
    return cudaGetLastError();
}

template <int L>
cudaError_t inv_launch_L(const DeviceTables& T, JobList<FinishJobX>& JL, FinishJobX* jobs, int n,
                         const FinishConsts& plain, const FinishConsts& split, cudaStream_t st) {
    if constexpr (L < 4) {
        return cudaErrorInvalidValue;  // rings below 16 finish in finish_fused_small_kernel
    } else {
        using S = RowShape<L>;
        const uint32_t ctas = assign_ctas<FinishJobX>(jobs, n, JL, [](const FinishJobX& j) -> uint64_t {
            return ((uint64_t)j.rows + S::ROWS - 1) / S::ROWS;
        });
        if (!ctas) return cudaSuccess;
        inv_rows_kernel<L><<<ctas, S::THREADS, S::SMEM, st>>>(JL, T.pc, plain, split, T.fwd, T.inv, T.inv_last);
    }
    return cudaGetLastError();
}

template <int L>
cudaError_t fused_launch_L(const DeviceTables& T, JobList<FinishJobX>& JL, FinishJobX* jobs, int n,
                           const FinishConsts& plain, const FinishConsts& split, cudaStream_t st) {
    if constexpr (L < 4) {
        const uint32_t ctas = assign_ctas<FinishJobX>(jobs, n, JL, [](const FinishJobX& j) -> uint64_t {
            return ((uint64_t)j.rows / kPrimes + kFusedSmallPolys - 1) / kFusedSmallPolys;
        });
        if (!ctas) return cudaSuccess;
        finish_fused_small_kernel<L><<<ctas, kFusedSmallPolys * kPrimes, 0, st>>>(JL, T.pc, T.cc, plain, split, T.fwd,
                                                                                  T.inv);
        return cudaGetLastError();
    } else if constexpr (L > 10) {
        return cudaErrorInvalidValue;
    } else {
        using S = FusedShape<L>;
        const uint32_t ctas = assign_ctas<FinishJobX>(jobs, n, JL, [](const FinishJobX& j) -> uint64_t {
            return ((uint64_t)j.rows / kPrimes + S::P - 1) / S::P;
        });
        if (!ctas) return cudaSuccess;
        finish_fused_kernel<L><<<ctas, S::THREADS, S::SMEM, st>>>(JL, T.pc, T.cc, plain, split, T.fwd, T.inv,
                                                                  T.inv_last);
        return cudaGetLastError();
    }
}

#define DM_DISPATCH_L(L, CALL)                                                                                 \
    switch (L) {                                                                                               \
        case 0: return CALL(0);                                                                                \
        case 1: return CALL(1);                                                                                \
        case 2: return CALL(2);                                                                                \
        case 3: return CALL(3);                                                                                \
        case 4: return CALL(4);                                                                                \
        case 5: return CALL(5);                                                                                \
        case 6: return CALL(6);                                                                                \
        case 7: return CALL(7);                                                                                \
        case 8: return CALL(8);                                                                                \
        case 9: return CALL(9);                                                                                \
        case 10: return CALL(10);                                                                              \
        case 11: return CALL(11);                                                                              \
        case 12: return CALL(12);                                                                              \
        case 13: return CALL(13);                                                                              \
    }

}  // namespace

cudaError_t upload_tables(DeviceTables* out) {
    const HostTables& H = host_tables();
    out->pc = H.pc;
    out->cc = H.cc;
    const std::vector<Tw>* src[4] = {&H.fwd, &H.inv, &H.fwd_last, &H.inv_last};
    Tw* dst[4] = {nullptr, nullptr, nullptr, nullptr};
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 4 && e == cudaSuccess; ++i) {
        const size_t bytes = sizeof(Tw) * src[i]->size();
        e = cudaMalloc(&dst[i], bytes);
        if (e == cudaSuccess) e = cudaMemcpy(dst[i], src[i]->data(), bytes, cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        for (Tw* d : dst)
            if (d) cudaFree(d);
        return e;
    }
    out->fwd = dst[0];
    out->inv = dst[1];
    out->fwd_last = dst[2];
    out->inv_last = dst[3];
    return cudaSuccess;
}

void free_tables(DeviceTables* t) {
    for (const Tw* d : {t->fwd, t->inv, t->fwd_last, t->inv_last})
        if (d) cudaFree(const_cast<Tw*>(d));
    t->fwd = t->inv = t->fwd_last = t->inv_last = nullptr;
}

cudaError_t launch_ntt_jobs(const DeviceTables& T, NttJob* jobs, int n, uint32_t L, cudaStream_t st, int group,
                            int elems) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs || L > (uint32_t)kLogMaxProverRing || (group != 32 && group != 64) || (elems != 16 && elems != 32))
        return cudaErrorInvalidValue;
    JobList<NttJob> JL;
#define DM_NTT_CALL(l) ntt_launch_L<l>(T, JL, jobs, n, st, group, elems)
    DM_DISPATCH_L(L, DM_NTT_CALL)
#undef DM_NTT_CALL
    return cudaErrorInvalidValue;
}

// Jobs of any ring sizes share a launch: each job's blocks cover its own rows and
// slots; blocks are 128 threads unless every job's rows are shorter.
namespace {
template <class Slots>
cudaError_t mac_launch_common(MacJobX* jobs, int n, Slots slots_of, JobList<MacJobX>& JL, uint64_t* total,
                              unsigned* bx, bool coords = false) {
    uint32_t widest = 1;
    *total = 0;
    JL.n = n;
    for (int i = 0; i < n; ++i) {
        if (jobs[i].L > (uint32_t)kLogMaxProverRing) return cudaErrorInvalidValue;
        const uint32_t slots = slots_of(jobs[i]);
        if (slots == 0) return cudaErrorInvalidValue;
        const uint32_t kc = coords && jobs[i].kc ? jobs[i].kc : 1u;
        if (kc != 1 && kc != 2 && kc != 4 && kc != 8) return cudaErrorInvalidValue;
        jobs[i].cta0 = (uint32_t)*total;
        JL.j[i] = jobs[i];
        *total += (uint64_t)((slots + kMacThreads - 1) / kMacThreads) * (kRows / kc) * jobs[i].parts;
        widest = slots > widest ? slots : widest;
    }
    *bx = widest < (uint32_t)kMacThreads ? widest : kMacThreads;
    return cudaSuccess;
}
}  // namespace

cudaError_t launch_mac_triple_jobs(const DeviceTables& T, MacJobX* jobs, int n, cudaStream_t st, int* kernels) {
    if (kernels) *kernels = 0;
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs) return cudaErrorInvalidValue;
    JobList<MacJobX> JL;
    uint64_t total;
    unsigned bx;
    // one launch per coordinates-per-thread value present
    for (uint32_t kc : {1u, 2u, 4u}) {
        MacJobX group[kMaxJobs];
        int m = 0;
        for (int i = 0; i < n; ++i) {
            const uint32_t jkc = jobs[i].kc ? jobs[i].kc : 1u;
            if (jkc != 1 && jkc != 2 && jkc != 4) return cudaErrorInvalidValue;
            if (jkc == kc) group[m++] = jobs[i];
        }
        if (!m) continue;
        cudaError_t e = mac_launch_common(group, m, [](const MacJobX& j) { return j.L ? 1u << (j.L - 1) : 0u; },
                                          JL, &total, &bx, true);  // slot pairs
        if (e != cudaSuccess) return e;
        if (!total) continue;
        switch (kc) {
            case 1: mac_triple_jobs_kernel<1><<<(unsigned)total, bx, 0, st>>>(JL, T.pc); break;
            case 2: mac_triple_jobs_kernel<2><<<(unsigned)total, bx, 0, st>>>(JL, T.pc); break;
            default: mac_triple_jobs_kernel<4><<<(unsigned)total, bx, 0, st>>>(JL, T.pc); break;
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        if (kernels) ++*kernels;
    }
    return cudaSuccess;
}

cudaError_t launch_mac_jobs(const DeviceTables& T, MacJobX* jobs, int n, bool split, cudaStream_t st, int* kernels) {
    if (kernels) *kernels = 0;
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs) return cudaErrorInvalidValue;
    JobList<MacJobX> JL;
    uint64_t total;
    unsigned bx;
    if (!split) {
        cudaError_t e = mac_launch_common(jobs, n, [](const MacJobX& j) { return 1u << j.L; }, JL, &total, &bx);
        if (e != cudaSuccess || !total) return e;
        mac_jobs_kernel<<<(unsigned)total, bx, 0, st>>>(JL, T.pc);
        if (kernels) *kernels = 1;
        return cudaGetLastError();
    }
    // one launch per coordinates-per-thread value present
    for (uint32_t kc : {1u, 2u, 4u, 8u}) {
        MacJobX group[kMaxJobs];
        int m = 0;
        for (int i = 0; i < n; ++i) {
            const uint32_t jkc = jobs[i].kc ? jobs[i].kc : 1u;
            if (jkc != 1 && jkc != 2 && jkc != 4 && jkc != 8) return cudaErrorInvalidValue;
            if (jkc == kc) group[m++] = jobs[i];
        }
        if (!m) continue;
        cudaError_t e = mac_launch_common(group, m, [](const MacJobX& j) { return j.L ? 1u << (j.L - 1) : 0u; }, JL,
                                          &total, &bx, true);
        if (e != cudaSuccess) return e;
        if (!total) continue;
        switch (kc) {
            case 1: mac_split_jobs_kernel<1><<<(unsigned)total, bx, 0, st>>>(JL, T.pc); break;
            case 2: mac_split_jobs_kernel<2><<<(unsigned)total, bx, 0, st>>>(JL, T.pc); break;
            case 4: mac_split_jobs_kernel<4><<<(unsigned)total, bx, 0, st>>>(JL, T.pc); break;
            default: mac_split_jobs_kernel<8><<<(unsigned)total, bx, 0, st>>>(JL, T.pc); break;
        }
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
        if (kernels) ++*kernels;
    }
    return cudaSuccess;
}

cudaError_t launch_finish_jobs(const DeviceTables& T, FinishJobX* jobs, int n, uint32_t L, cudaStream_t st) {
    if (n <= 0) return cudaSuccess;
    if (n > kMaxJobs || L > (uint32_t)kLogMaxProverRing) return cudaErrorInvalidValue;
    for (int i = 0; i < n; ++i)
        if (jobs[i].parts == 0 || jobs[i].parts > kMaxMacParts || (jobs[i].rhs && jobs[i].parts != 1))
            return cudaErrorInvalidValue;
    const HostTables& H = host_tables();
    FinishConsts plain, split;
    for (int i = 0; i < kPrimes; ++i) {
        plain.f[i] = H.ninv[i][L];
        plain.fs[i] = H.ninvs[i][L];
        split.f[i] = H.ninv4[i][L];
        split.fs[i] = H.ninv4s[i][L];
    }
    if (L <= 10) {
        JobList<FinishJobX> JL;
#define DM_FUSED_CALL(l) fused_launch_L<l>(T, JL, jobs, n, plain, split, st)
        DM_DISPATCH_L(L, DM_FUSED_CALL)
#undef DM_FUSED_CALL
        return cudaErrorInvalidValue;
    }
    cudaError_t e = cudaErrorInvalidValue;
    {
        JobList<FinishJobX> JL;
#define DM_INV_CALL(l) inv_launch_L<l>(T, JL, jobs, n, plain, split, st)
        auto inv = [&]() -> cudaError_t {
            DM_DISPATCH_L(L, DM_INV_CALL)
            return cudaErrorInvalidValue;
        };
#undef DM_INV_CALL
        e = inv();
    }
    if (e != cudaSuccess) return e;
    JobList<FinishJobX> JC;
    const uint32_t Lc = L;
    uint64_t total = 0;
    JC.n = n;
    for (int i = 0; i < n; ++i) {
        JC.j[i] = jobs[i];
        JC.j[i].cta0 = (uint32_t)total;
        total += ((((uint64_t)jobs[i].rows / kPrimes) << Lc) + kCrtThreads - 1) / kCrtThreads;
    }
    if (!total) return cudaSuccess;
    crt_jobs_kernel<<<(unsigned)total, kCrtThreads, 0, st>>>(JC, L, T.pc, T.cc);
    return cudaGetLastError();
}

}  // namespace dm
