// Multi-job kernel interfaces.  Every kernel here takes a list of jobs, so one
// launch serves one request (the plain path) or the same stage of many requests
// (the batched and serving paths coalesce same-degree rounds into one launch).
#pragma once

#include <cuda_runtime.h>

#include "dm_kernels.cuh"

namespace dm {

constexpr int kMaxJobs = 48;
// Column splits of one multiply-accumulate.  The finish sums a row's parts with
// plain 32-bit adds: 16 residues below 2^28 cannot overflow.
constexpr uint32_t kMaxMacParts = 16;

// Launch-shape knobs (set per context; defaults are the built-in choices, an
// autotuner measures and overrides them per ring size).
enum TuneKnob : int {
    kTuneNttGroup = 0,   // threads per block of the forward transform for rings of 2^L < 2^10: 32 or 64
    kTuneMacTriple = 1,  // resident blocks per SM a triple MAC's column split fills: 1..32
    kTuneMacSplit = 2,   // the same for the split MAC
    kTuneMacPlain = 3,   // the same for the single-sum MAC
    kTuneSplitCoords = 4,   // commitment coordinates per thread of the split MAC: 1, 2, 4 or 8
    kTuneTripleCoords = 5,  // the same for the triple MAC: 1, 2 or 4
    kTuneNttRadix = 6,      // residues per thread of the forward transform (pass radix): 16 or 32
    kTuneKnobs = 7,
};
constexpr int kTuneDefault[kTuneKnobs] = {64, 8, 8, 8, 1, 1, 16};
// Built-in value of a knob at ring 2^L: kTuneDefault, except eight coordinates
// per thread for the split MAC from rings of 2^9 on (measured 20-26 % faster than
// one there on GB300, and 2-9 % faster than four; within noise below 2^9).
constexpr int tune_default(int knob, int L) { return knob == kTuneSplitCoords && L >= 9 ? 8 : kTuneDefault[knob]; }
static_assert((uint64_t)kMaxMacParts * ((1u << 28) - 1) < (1ull << 32), "part sums fit 32 bits");

// ---- forward NTT: coefficients [npolys][2^L] -> residues [npolys][9][2^L] ----
struct NttJob {
    const uint4* src;
    uint32_t* dst;
    uint32_t npolys;
    uint32_t cta0;  // filled by the launcher
};

// ---- multiply-accumulate over columns (all jobs of a launch share L) ----
// plain: partials[part][k*9+p][slot] = sum_{i<count} G[g_base+i][k][p][slot] * M[m_base+i][p][slot]
// split: chk over 2^L slots, lp / rp over 2^(L-1) (even/odd cross terms)
struct MacJobX {
    const uint32_t* G;
    const uint32_t* M;
    uint32_t* out0;  // plain: partials; split: chk partials
    uint32_t* out1;  // split: lp partials
    uint32_t* out2;  // split: rp partials
    uint32_t g_base, m_base, count, parts;
    uint32_t cta0;
    // Triple MAC only: 0 = column pairs (i, i + count); otherwise pairs
    // (i, i + pair) for i < count <= pair with every witness column from `pair`
    // on zero, so the witness is read at i only and R is zero.
    uint32_t pair;
    uint32_t L;  // ring size 2^L of this job (jobs of any sizes share a launch)
    // Split and triple MACs: commitment coordinates per thread, 1, 2, 4 (or 8,
    // split only); 0 reads as 1.  A thread then loads each witness slot pair
    // once for kc generator rows, and a part covers kRows / kc rows.
    uint32_t kc;
};

// ---- sum partials, inverse NTT, CRT to Z_q, optional compare (all jobs share L) ----
enum FinishMode : uint32_t { kFinishPlain = 0, kFinishSplitL = 1, kFinishSplitR = 2 };
// partials: [parts][rows][2^L] residues, rows = npolys * 9 (coordinate-major:
// row = poly * 9 + prime).  The inverse transform writes its residues over part
// 0 (each row belongs to one block), then the CRT reads them back.
struct FinishJobX {
    uint32_t* partials;
    uint4* out;            // [npolys][2^L]
    const uint4* expect;   // compared with out when non-null
    uint32_t* flag;        // set to 1 on mismatch (a plain store: device or mapped pinned host memory)
    uint32_t parts;
    uint32_t mode;         // FinishMode
    uint32_t rows;         // npolys * kPrimes
    uint32_t cta0;         // filled by the launcher
    // When set (with parts == 1): the row's input is the slotwise product of the
    // transformed rows `partials` and `rhs` (a negacyclic ring product per
    // polynomial) instead of a sum of partials.
    const uint32_t* rhs;
    // When set: a second copy of out in mapped pinned host memory (same layout),
    // written by the kernel itself, so the host reads the stage's commitments
    // once the stream has passed the kernel, without a device-to-host copy.
    uint4* host_out;
};

// ---- folds and commitment algebra in the coefficient domain ----
enum FoldMode : uint32_t {
    kFoldVec = 0,       // dst[e] = a[e] + x * b[e]
    kFoldPoly = 1,      // dst[poly][j] = a[poly][2j] + x * a[poly][2j+1]
    kFoldPolyX = 2,     // dst[poly][j] = a[poly][2j] + x * (X * odd)[j]
    kCombine = 3,       // dst[e] = a[e] + x * b[e] + y * c[e]
    kCombineEven = 4,   // dst[k][j] = a[k][2j] + x * b[k][j] + y * c[k][j]
    kCanon = 5,         // dst[e] = a[e] mod q
};
struct FoldJob {
    uint4* dst;
    const uint4* a;
    const uint4* b;
    const uint4* c;
    fq x, y;
    uint64_t n;     // output elements
    uint32_t mode;
    uint32_t Lout;  // log2 of the output polynomial length (poly modes, combine_even)
    uint32_t cta0;
};

// ---- hashing / expansion ----
struct GenJob {
    uint32_t key[8];
    uint4* dst;
    uint64_t total;  // N * 8 * 2^log_n
    uint32_t log_n;
    uint32_t cta0;
};
struct UnpackJob {
    const uint8_t* file;
    uint64_t len;
    uint4* dst;
    uint64_t total;
    uint32_t cta0;
};
struct HashJob {
    const uint8_t* file;
    uint64_t len;
    uint32_t* scratch;  // 2 * 8 * nchunks words
    uint32_t* out8;
    uint32_t cta0;
};

// group: threads per block for rings below 2^10 (32 or 64, kTuneNttGroup)
// elems: residues per thread, i.e. the pass radix (16, or 32 for rings of 2^5
// and up: radix-32 passes, one exchange fewer at 2^9 and 2^10; kTuneNttRadix)
cudaError_t launch_ntt_jobs(const DeviceTables& T, NttJob* jobs, int n, uint32_t L, cudaStream_t st, int group = 64,
                            int elems = 16);
// kernels (optional): how many kernels it launched (the split MAC launches one
// per coordinates-per-thread value among the jobs)
cudaError_t launch_mac_jobs(const DeviceTables& T, MacJobX* jobs, int n, bool split, cudaStream_t st,
                            int* kernels = nullptr);
// Triple MAC (count = h column pairs): out0 = full sum, out1 = L, out2 = R.
// kernels (optional): how many kernels it launched (one per kc value among the jobs)
cudaError_t launch_mac_triple_jobs(const DeviceTables& T, MacJobX* jobs, int n, cudaStream_t st,
                                   int* kernels = nullptr);
cudaError_t launch_finish_jobs(const DeviceTables& T, FinishJobX* jobs, int n, uint32_t L, cudaStream_t st);  // 2 launches
cudaError_t launch_fold_jobs(FoldJob* jobs, int n, cudaStream_t st);
cudaError_t launch_gen_jobs(GenJob* jobs, int n, cudaStream_t st);
cudaError_t launch_unpack_jobs(UnpackJob* jobs, int n, cudaStream_t st);
cudaError_t launch_hash_jobs(HashJob* jobs, int n, cudaStream_t st);  // 2 launches

}  // namespace dm
