#include "proof.h"

#include <chrono>

#include <cstring>

#include "dm_nvtx.h"
#include "host_blake3.h"

namespace dm {

namespace {

// Commitment slots in comm_ (each 8 * S elements).
enum Slot { kC = 0, kL = 1, kR = 2, kCt = 3, kV = 4, kLp = 5, kRp = 6, kChk = 7, kSlots = 8 };
constexpr uint32_t kMaxParts = kMaxMacParts;
// Pinned tail after the three commitment slots: [0,32) file id, [32,40) check
// flags, [48,64) m*.  The file id and the flags are written there by the kernels
// (mapped pinned memory), like the commitments of small rings that the finishes
// mirror into the slots, so such a stage needs no device-to-host copy; m* is
// copied once per proof.
constexpr size_t kTail = 128;

constexpr uint32_t kRows = kRank * kPrimes;  // MAC rows per job: (coordinate, prime)

void unpack_module(const uint8_t* src, uint32_t n, Module& m) {
    m.n = n;
    m.c.resize((size_t)kRank * n);
    const uint4* p = reinterpret_cast<const uint4*>(src);
    for (size_t i = 0; i < m.c.size(); ++i) m.c[i] = fq{{p[i].x, p[i].y, p[i].z, p[i].w}};
}

template <class J>
int launch_chunks(std::vector<J>& v, cudaError_t (*fn)(J*, int, cudaStream_t), cudaStream_t st, int per_launch,
                  int* launches) {
    for (size_t i = 0; i < v.size(); i += kMaxJobs) {
        const int n = (int)std::min<size_t>(kMaxJobs, v.size() - i);
        cudaError_t e = fn(v.data() + i, n, st);
        if (e != cudaSuccess) return (int)e;
        *launches += per_launch;
    }
    return 0;
}

}  // namespace

// ============================================================== Plan

void Plan::clear() {
    hash.clear();
    unpack.clear();
    mac.clear();
    split.clear();
    triple.clear();
    gen.clear();
    fold.clear();
    for (int L = 0; L <= kLogMaxProverRing; ++L) {
        ntt[L].clear();
        finish[L].clear();
    }
    d2h.clear();
    wait_events.clear();
    record_events.clear();
    fills.clear();
}

bool Plan::empty() const {
    if (!hash.empty() || !unpack.empty() || !gen.empty() || !fold.empty() || !mac.empty() || !split.empty() ||
        !triple.empty())
        return false;
    for (int L = 0; L <= kLogMaxProverRing; ++L)
        if (!ntt[L].empty() || !finish[L].empty())
            return false;
    return d2h.empty();
}

int Plan::launch(Context* ctx, cudaStream_t st, std::string* err) {
    const int n = launch_all(ctx, st, err);
    for (auto& f : fills) {
        if (n < 0) ctx->prover_cache()->poison(f);
        else ctx->prover_cache()->publish(f);
    }
    return n;
}

int Plan::launch_all(Context* ctx, cudaStream_t st, std::string* err) {
    const DeviceTables& T = ctx->tables();
    int launches = 0;
    for (cudaEvent_t e : wait_events) {
        const cudaError_t we = cudaStreamWaitEvent(st, e, 0);
        if (we != cudaSuccess) {
            *err = std::string("wait for a cached generator family: ") + cudaGetErrorString(we);
            return kECuda;
        }
    }
    const bool prof = ctx->profiling();
    auto timed = [&](const char* name, double bytes, double ops, auto&& body) -> int {
        cudaEvent_t a = nullptr;
        if (prof) {
            a = ctx->take_event();
            cudaEventRecord(a, st);
        }
        const int before = launches;
        NvtxRange range(name);
        const int rc = body();
        if (rc != 0) {
            *err = std::string(name) + ": " + cudaGetErrorString((cudaError_t)rc);
            return kECuda;
        }
        if (a) {
            cudaEvent_t b = ctx->take_event();
            cudaEventRecord(b, st);
            ctx->record(name, a, b, bytes, ops, launches - before, st);
        }
        return 0;
    };
    int rc;
    if (!hash.empty()) {
        double bytes = 0, ops = 0;
        for (auto& j : hash) {
            bytes += (double)j.len;
            ops += (double)((j.len + 63) / 64 + (j.len + 1023) / 1024);
        }
        if ((rc = timed("file_hash", bytes, ops, [&] { return launch_chunks(hash, launch_hash_jobs, st, 2, &launches); })))
            return rc;
    }
    if (!unpack.empty()) {
        double bytes = 0;
        for (auto& j : unpack) bytes += (double)j.len + (double)j.total * 16;
        if ((rc = timed("unpack_witness", bytes, 0,
                        [&] { return launch_chunks(unpack, launch_unpack_jobs, st, 1, &launches); })))
            return rc;
    }
    if (!gen.empty()) {
        double bytes = 0, ops = 0;
        for (auto& j : gen) {
            bytes += (double)j.total * 16;
            ops += (double)j.total;
        }
        if ((rc = timed("gen_generators", bytes, ops, [&] { return launch_chunks(gen, launch_gen_jobs, st, 1, &launches); })))
            return rc;
    }
    if (!fold.empty()) {
        double bytes = 0;
        for (auto& j : fold) bytes += (double)j.n * (j.mode == kCombine || j.mode == kCombineEven ? 64 : 48);
        if ((rc = timed("fold", bytes, 0, [&] { return launch_chunks(fold, launch_fold_jobs, st, 1, &launches); })))
            return rc;
    }
    for (int L = 0; L <= kLogMaxProverRing; ++L) {
        if (ntt[L].empty()) continue;
        double polys = 0;
        for (auto& j : ntt[L]) polys += j.npolys;
        const double bytes = polys * (double)(1u << L) * (16 + 4 * kPrimes);  // 16 B read + 9 residues written
        const double ops = polys * (double)kPrimes * (double)(1u << L) / 2 * L;  // butterflies
        if ((rc = timed("ntt_fwd", bytes, ops, [&] {
                 for (size_t i = 0; i < ntt[L].size(); i += kMaxJobs) {
                     const int n = (int)std::min<size_t>(kMaxJobs, ntt[L].size() - i);
                     cudaError_t e = launch_ntt_jobs(T, ntt[L].data() + i, n, (uint32_t)L, st,
                                                     ctx->tuning(kTuneNttGroup, (uint32_t)L),
                                                     ctx->tuning(kTuneNttRadix, (uint32_t)L));
                     if (e != cudaSuccess) return (int)e;
                     ++launches;
                 }
                 return 0;
             })))
            return rc;
    }
    for (int pass = 0; pass < 3; ++pass) {
        auto& v = pass == 0 ? mac : (pass == 1 ? split : triple);
        if (v.empty()) continue;
        // columns read: count (plain, split) or 2 * count (triple pairs)
        const double cols_per_count = pass == 2 ? 2.0 : 1.0;
        const double macs_per_col = pass == 0 ? 1.0 : 2.0;
        double macs = 0, bytes = 0;
        for (auto& j : v) {
            const double cols = (double)j.count * cols_per_count;
            macs += cols * (double)kRows * (double)(1u << j.L) * macs_per_col;
            // G residues (4 B per column, coordinate, prime, slot) + M residues (shared by 8 coordinates)
            bytes += cols * (double)(1u << j.L) * (kRows * 4.0 + kPrimes * 4.0);
        }
        const char* name = pass == 0 ? "mac" : (pass == 1 ? "mac_split" : "mac");
        if ((rc = timed(name, bytes, macs, [&] {
                 for (size_t i = 0; i < v.size(); i += kMaxJobs) {
                     const int n = (int)std::min<size_t>(kMaxJobs, v.size() - i);
                     int k = 1;
                     cudaError_t e = pass == 2 ? launch_mac_triple_jobs(T, v.data() + i, n, st, &k)
                                               : launch_mac_jobs(T, v.data() + i, n, pass == 1, st, &k);
                     if (e != cudaSuccess) return (int)e;
                     launches += k;
                 }
                 return 0;
             })))
            return rc;
    }
    for (int L = kLogMaxProverRing; L >= 0; --L) {
        if (finish[L].empty()) continue;
        double bytes = 0;
        for (auto& j : finish[L]) bytes += ((double)j.parts + 2.0) * j.rows * (1u << L) * 4 + (j.rows / kPrimes) * (1u << L) * 16.0;
        if ((rc = timed("finish", bytes, 0, [&] {
                 for (size_t i = 0; i < finish[L].size(); i += kMaxJobs) {
                     const int n = (int)std::min<size_t>(kMaxJobs, finish[L].size() - i);
                     cudaError_t e = launch_finish_jobs(T, finish[L].data() + i, n, (uint32_t)L, st);
                     if (e != cudaSuccess) return (int)e;
                     launches += L <= 10 ? 1 : 2;  // the fused finish, or inverse transform + CRT
                 }
                 return 0;
             })))
            return rc;
    }
    for (cudaEvent_t e : record_events) {
        const cudaError_t re = cudaEventRecord(e, st);
        if (re != cudaSuccess) {
            *err = std::string("record a cached generator family: ") + cudaGetErrorString(re);
            return kECuda;
        }
    }
    for (auto& c : d2h) {
        cudaError_t e = cudaMemcpyAsync(c.dst, c.src, c.bytes, cudaMemcpyDeviceToHost, st);
        if (e != cudaSuccess) {
            *err = std::string("device-to-host copy: ") + cudaGetErrorString(e);
            return kECuda;
        }
    }
    return launches;
}

// ============================================================== ProofState

uint64_t ProofState::footprint(uint64_t len) {
    uint32_t d;
    uint64_t S;
    if (!square_layout_for_byte_len(len, &d, &S)) return ~0ull;
    const uint64_t S2 = S * S;
    auto r = [](uint64_t b) { return (b + 255) & ~255ull; };
    return r(len + 16) + r(file_hash_scratch_words(len) * 4) + r(S2 * 16) + r(S2 / 2 * 16) + r(8 * S2 * 16) +
           r(4 * S2 * 16) + r(S2 * kPrimes * 4) + r(8 * S2 * kPrimes * 4) + r(3ull * kMaxParts * kRows * S * 4) +
           r((uint64_t)kSlots * kRank * S * 16);
}

const uint4* ProofState::g_round0() const { return cached_.g ? cached_.g : g_a_.as<uint4>(); }

void ProofState::release() {
    if (cached_.entry) {
        // a request ends only after its last stage's copies landed: nothing of it
        // still reads the entry
        ctx_->prover_cache()->release(cached_);
        cached_ = ProverGenCache::Ref{};
    }
    DevMem* all[] = {&file_, &hash_scratch_, &m_a_, &m_b_, &g_a_, &g_b_, &mhat_, &ghat_, &partials_, &comm_};
    for (DevMem* m : all) m->reset();
    if (pinned_) ctx_->put_pinned(pinned_, pinned_bytes_);
    pinned_ = nullptr;
}

ProofState::~ProofState() { release(); }

int ProofState::fail(int code, const std::string& msg) {
    stage_ = Stage::Failed;
    err_ = msg;
    err_code_ = code;
    return code;
}

uint32_t ProofState::stage_L() const {
    if (stage_ == Stage::Init) return d_;
    if (stage_ == Stage::Vec) return d_ - (uint32_t)round_;
    if (stage_ == Stage::Poly) return d_ - (uint32_t)round_ - 1;
    return 0;
}

bool ProofState::opening(fq* out) const {
    if (!have_opening_) return false;
    *out = opening_;
    return true;
}

int ProofState::setup(const uint8_t* file, uint64_t len, bool on_device, const uint8_t seed[32],
                      const uint8_t epoch[32], uint64_t max_preprocess_bytes, cudaStream_t stream) {
    uint32_t d;
    uint64_t S;
    if (!square_layout_for_byte_len(len, &d, &S)) return fail(kEInval, "square witness dimension overflow");
    const uint64_t est = S * S * 16 * 2;  // io.rs:42-49
    if (est > max_preprocess_bytes)
        return fail(kEInval, "full witness expansion requires " + std::to_string(est) +
                                 " bytes, above max_preprocess_bytes=" + std::to_string(max_preprocess_bytes) +
                                 "; split the file into smaller statements");
    if (d > (uint32_t)kMaxDepth)
        return fail(kEUnsupported,
                    "fold depth " + std::to_string(d) + " exceeds the supported maximum " + std::to_string(kMaxDepth));
    if (len > 0 && file == nullptr) return fail(kEInval, "null file buffer");
    d_ = d;
    S_ = N_ = n_ = (uint32_t)S;
    len_ = len;
    mcols_ = (uint32_t)((coeff_count_for_byte_len(len) + S - 1) / S);
    alloc_stream_ = stream;
    std::memcpy(seed_, seed, 32);
    const uint64_t S2 = S * S;
    int rc = kOk;
    auto need = [&](DevMem& m, size_t bytes) {
        if (rc == kOk) rc = m.alloc(ctx_, bytes, stream);
    };
    for (int attempt = 0; attempt < 2; ++attempt) {
        rc = kOk;
        if (!on_device) need(file_, len + 16);
        need(hash_scratch_, file_hash_scratch_words(len) * 4);
        need(m_a_, S2 * 16);
        need(m_b_, S2 / 2 * 16);
        need(g_a_, 8 * S2 * 16);
        need(g_b_, 4 * S2 * 16);
        need(mhat_, S2 * kPrimes * 4);
        need(ghat_, 8 * S2 * kPrimes * 4);
        need(partials_, 3ull * kMaxParts * kRows * S * 4);
        need(comm_, (uint64_t)kSlots * kRank * S * 16);
        if (rc == kOk || !ctx_->prover_cache()) break;
        // the budget is held by cached generator families: drop unreferenced ones, once
        release();
        if (!ctx_->prover_cache()->trim(footprint(len))) break;
    }
    if (rc != kOk) return fail(rc, "HBM budget exhausted allocating prover state (" + std::to_string(footprint(len)) + " bytes)");
    pinned_bytes_ = 3ull * kRank * S * 16 + kTail;
    pinned_ = static_cast<uint8_t*>(ctx_->get_pinned(pinned_bytes_));
    if (!pinned_) return fail(kECuda, "cudaMallocHost failed");
    // the check flags start clear (kernels only ever set them); no kernel of this
    // request has been launched yet, and the buffer's previous owner has finished
    std::memset(pinned_ + 3ull * kRank * S * 16, 0, kTail);
    d_file_ = on_device ? file : file_.as<uint8_t>();
    if (!on_device && len) {
        cudaError_t e = cudaMemcpyAsync(file_.as<uint8_t>(), file, len, cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess) return fail(kECuda, std::string("H2D file: ") + cudaGetErrorString(e));
    }
    blake3_keyed_hash(seed, "g0", 2, st_.g_0_seed);  // sis.rs:70, 208-210
    st_.original_len_bytes = len;
    st_.d = d;
    std::memcpy(epoch_copy_, epoch, 32);  // the transcript is keyed after the Init stage yields the file id
    stage_ = Stage::Init;
    return kOk;
}

// Transforms and the multiply-accumulate of a commitment stage over `cols`
// columns of ring 2^L of which the first `c` can be nonzero: the full sum into
// `part`, and for cols >= 2 the cross terms L (pairs (i, i + cols/2)) and R.
// With c <= cols/2 the witness half from cols/2 on is zero: only c witness
// columns and the generator columns [0, c) and [cols/2, cols/2 + c) are
// transformed and read, and R is zero.  Returns whether the cross terms exist.
bool ProofState::plan_commit(Plan& P, uint32_t L, uint32_t cols, uint32_t c, const uint4* m_src, const uint4* g_src,
                             uint32_t* part, uint32_t* ghat, bool g_transformed) {
    const uint64_t s = 1ull << L;
    uint32_t* mh = mhat_.as<uint32_t>();
    uint32_t* gh = ghat ? ghat : ghat_.as<uint32_t>();
    const uint64_t gcol_in = 8 * s, gcol_out = 8 * (uint64_t)kPrimes * s;  // one generator column
    auto ntt = [&](const uint4* src, uint32_t* dst, uint64_t polys) {
        // generator columns that are already in `ghat` (a cached family) are not transformed again
        if (polys && !(g_transformed && dst != mh)) P.ntt[L].push_back(NttJob{src, dst, polys, 0});
    };
    if (cols < 2) {
        ntt(m_src, mh, c);
        ntt(g_src, gh, 8ull * c);
        parts_ = ctx_->mac_parts(kTuneMacPlain, L, (uint32_t)s, c);
        P.mac.push_back(MacJobX{gh, mh, part, nullptr, nullptr, 0, 0, c, parts_, 0, 0, L});
        return false;
    }
    const uint32_t half = cols / 2;
    const uint32_t kc = (uint32_t)ctx_->tuning(kTuneTripleCoords, L);
    const int bps = ctx_->tuning(kTuneMacTriple, L);
    if (c <= half) {
        ntt(m_src, mh, c);
        ntt(g_src, gh, 8ull * c);
        ntt(g_src + half * gcol_in, gh + half * gcol_out, 8ull * c);
        parts_ = ctx_->mac_parts_for(bps, (uint32_t)(s / 2), c, kRows / kc);
        const size_t ps = (size_t)parts_ * kRows * s;
        P.triple.push_back(MacJobX{gh, mh, part, part + ps, part + 2 * ps, 0, 0, c, parts_, 0, half, L, kc});
    } else {
        ntt(m_src, mh, cols);
        ntt(g_src, gh, 8ull * cols);
        parts_ = ctx_->mac_parts_for(bps, (uint32_t)(s / 2), half, kRows / kc);
        const size_t ps = (size_t)parts_ * kRows * s;
        P.triple.push_back(MacJobX{gh, mh, part, part + ps, part + 2 * ps, 0, 0, half, parts_, 0, 0, L, kc});
    }
    return true;
}

void ProofState::plan_stage(Plan& P) {
    const uint32_t S = S_;
    const size_t slot = (size_t)kRank * S;
    uint4* C = comm_.as<uint4>();
    auto cs = [&](int i) { return C + (size_t)i * slot; };
    uint32_t* part = partials_.as<uint32_t>();
    uint8_t* tail = pinned_ + 3 * slot * 16;
    uint32_t* flags = reinterpret_cast<uint32_t*>(tail + 32);
    // The three commitment slots the host reads after a stage.  Up to rings of
    // 2^(kCopyFromL - 1) the finishes mirror them into pinned host memory (no copy
    // to issue, which is what the small, latency-bound stages pay for); from
    // 2^kCopyFromL on (64 KiB slots and more; few, long stages) one copy per slot,
    // which keeps the finishes' stores on the device.
    constexpr uint32_t kCopyFromL = 9;
    const uint32_t Lout = stage_ == Stage::Init ? d_ : (stage_ == Stage::Vec ? d_ - (uint32_t)round_
                                                                                : d_ - (uint32_t)round_ - 1);
    const bool mapped = Lout < kCopyFromL;
    uint4* hm0 = mapped ? reinterpret_cast<uint4*>(pinned_) : nullptr;
    uint4* hm1 = mapped ? reinterpret_cast<uint4*>(pinned_ + slot * 16) : nullptr;
    uint4* hm2 = mapped ? reinterpret_cast<uint4*>(pinned_ + 2 * slot * 16) : nullptr;
    auto copy3 = [&](const uint4* s0, const uint4* s1, const uint4* s2, size_t n0, size_t n12) {
        if (mapped) return;
        P.d2h.push_back(Copy{pinned_, s0, n0 * 16});
        if (s1) P.d2h.push_back(Copy{pinned_ + slot * 16, s1, n12 * 16});
        if (s2) P.d2h.push_back(Copy{pinned_ + 2 * slot * 16, s2, n12 * 16});
    };
    auto fin = [](uint32_t* partials, uint4* out, const uint4* expect, uint32_t* flag, uint32_t parts, uint32_t mode,
                  uint4* host_out) {
        return FinishJobX{partials, out, expect, flag, parts, mode, kRows, 0, nullptr, host_out};
    };
    if (stage_ == Stage::Init) {
        const uint32_t L = d_;
        const uint64_t S2 = (uint64_t)S * S;
        P.hash.push_back(HashJob{d_file_, len_, hash_scratch_.as<uint32_t>(), reinterpret_cast<uint32_t*>(tail), 0});
        P.unpack.push_back(UnpackJob{d_file_, len_, m_a_.as<uint4>(), S2, 0});
        GenJob g{};
        for (int i = 0; i < 8; ++i)
            g.key[i] = (uint32_t)st_.g_0_seed[4 * i] | ((uint32_t)st_.g_0_seed[4 * i + 1] << 8) |
                       ((uint32_t)st_.g_0_seed[4 * i + 2] << 16) | ((uint32_t)st_.g_0_seed[4 * i + 3] << 24);
        g.dst = g_a_.as<uint4>();
        g.total = 8 * S2;
        g.log_n = L;
        ProverGenCache* cache = ctx_->prover_cache();
        cached_ = ProverGenCache::Ref{};
        if (cache && cache->acquire(st_.g_0_seed, L, &P, &cached_) == kOk) {
            if (cached_.fill) {
                // expand into the entry and transform every column (later holders
                // may have more nonzero witness columns than this file)
                g.dst = cached_.g;
                P.gen.push_back(g);
                P.ntt[L].push_back(NttJob{cached_.g, cached_.ghat, 8ull * S, 0});
                P.record_events.push_back(cached_.ready);
                P.fills.push_back(cached_);
            } else if (cached_.ready) {
                P.wait_events.push_back(cached_.ready);
            }
        } else {
            cached_ = ProverGenCache::Ref{};
            P.gen.push_back(g);
        }
        const bool nj = plan_commit(P, L, S, mcols_ < S ? mcols_ : S, m_a_.as<uint4>(), g_round0(), part,
                                    cached_.ghat, cached_.ghat != nullptr);
        if (nj) {
            const size_t pstride = (size_t)parts_ * kRows * S;
            P.finish[L].push_back(fin(part + pstride, cs(kL), nullptr, nullptr, parts_, kFinishPlain, hm1));
            P.finish[L].push_back(fin(part + 2 * pstride, cs(kR), nullptr, nullptr, parts_, kFinishPlain, hm2));
        }
        P.finish[L].push_back(fin(part, cs(kC), nullptr, nullptr, parts_, kFinishPlain, hm0));
        copy3(cs(kC), nj ? cs(kL) : nullptr, nj ? cs(kR) : nullptr, slot, slot);
        return;
    }
    const uint32_t L = d_ - (uint32_t)round_, s = 1u << L, h = s / 2;
    const uint64_t s2 = (uint64_t)s * s;
    if (stage_ == Stage::Vec) {
        P.fold.push_back(FoldJob{m_b_.as<uint4>(), m_a_.as<uint4>(), m_a_.as<uint4>() + (uint64_t)h * s, nullptr, x_,
                                 fq_zero(), (uint64_t)h * s, kFoldVec, 0});
        const uint4* gsrc = round_ == 0 ? g_round0() : g_a_.as<uint4>();
        P.fold.push_back(FoldJob{g_b_.as<uint4>(), gsrc, gsrc + 4 * s2, nullptr, xi_, fq_zero(), 4 * s2, kFoldVec, 0});
        P.fold.push_back(FoldJob{cs(kCt), cs(kC), cs(kL), cs(kR), xi_, x_, (uint64_t)kRank * s, kCombine, 0});
        // the folded witness has h columns, of which the first c can be nonzero:
        // the check and both cross terms only need those columns
        const uint32_t c = mcols_ < h ? mcols_ : h;
        if (c) {
            P.ntt[L].push_back(NttJob{m_b_.as<uint4>(), mhat_.as<uint32_t>(), c, 0});
            P.ntt[L].push_back(NttJob{g_b_.as<uint4>(), ghat_.as<uint32_t>(), 8ull * c, 0});
        }
        const uint32_t kc = (uint32_t)ctx_->tuning(kTuneSplitCoords, L);
        parts_ = ctx_->mac_parts_for(ctx_->tuning(kTuneMacSplit, L), h, c, kRows / kc);
        uint32_t* pchk = part;
        uint32_t* plp = part + (size_t)parts_ * kRows * s;
        uint32_t* prp = plp + (size_t)parts_ * kRows * h;
        P.split.push_back(
            MacJobX{ghat_.as<uint32_t>(), mhat_.as<uint32_t>(), pchk, plp, prp, 0, 0, c, parts_, 0, 0, L, kc});
        // The recomputed commitment V is checked against the folded one (Ct); the
        // host reads V's mirror as Ct, which it equals unless the check flag is set
        // (and then the stage fails before anything is absorbed).
        P.finish[L].push_back(fin(pchk, cs(kV), cs(kCt), flags, parts_, kFinishPlain, hm0));
        P.finish[L - 1].push_back(fin(plp, cs(kLp), nullptr, nullptr, parts_, kFinishSplitL, hm1));
        P.finish[L - 1].push_back(fin(prp, cs(kRp), nullptr, nullptr, parts_, kFinishSplitR, hm2));
        copy3(cs(kCt), cs(kLp), cs(kRp), (size_t)kRank * s, (size_t)kRank * h);
        return;
    }
    if (stage_ == Stage::Poly) {
        const uint32_t Ln = L - 1;
        const uint64_t h2 = (uint64_t)h * h;
        P.fold.push_back(FoldJob{m_a_.as<uint4>(), m_b_.as<uint4>(), nullptr, nullptr, y_, fq_zero(), h2, kFoldPoly, Ln, 0});
        P.fold.push_back(FoldJob{g_a_.as<uint4>(), g_b_.as<uint4>(), nullptr, nullptr, yi_, fq_zero(), 8 * h2, kFoldPolyX,
                                 Ln, 0});
        P.fold.push_back(FoldJob{cs(kC), cs(kCt), cs(kLp), cs(kRp), yi_, y_, (uint64_t)kRank * h, kCombineEven, Ln, 0});
        const bool nj = plan_commit(P, Ln, h, mcols_ < h ? mcols_ : h, m_a_.as<uint4>(), g_a_.as<uint4>(), part);
        if (nj) {
            const size_t pstride = (size_t)parts_ * kRows * h;
            P.finish[Ln].push_back(fin(part + pstride, cs(kL), nullptr, nullptr, parts_, kFinishPlain, hm1));
            P.finish[Ln].push_back(fin(part + 2 * pstride, cs(kR), nullptr, nullptr, parts_, kFinishPlain, hm2));
        }
        // as in the vector stage: the recomputed Chk's mirror is the folded C
        P.finish[Ln].push_back(fin(part, cs(kChk), cs(kC), flags + 1, parts_, kFinishPlain, hm0));
        copy3(cs(kC), nj ? cs(kL) : nullptr, nj ? cs(kR) : nullptr, (size_t)kRank * h, (size_t)kRank * h);
        if (round_ + 1 == d_) P.d2h.push_back(Copy{tail + 48, m_a_.as<uint4>(), 16});
    }
}

int ProofState::complete_stage() {
    const size_t slot = (size_t)kRank * S_;
    const uint8_t* tail = pinned_ + 3 * slot * 16;
    uint32_t fl[2];
    std::memcpy(fl, tail + 32, 8);
    if (stage_ == Stage::Init) {
        std::memcpy(st_.file_id, tail, 32);
        tr_ = Transcript(epoch_copy_, st_.file_id);
        unpack_module(pinned_, S_, st_.com_0);
        current_ = st_.com_0;
        if (S_ >= 2) {
            unpack_module(pinned_ + slot * 16, S_, pend_l_);
            unpack_module(pinned_ + 2 * slot * 16, S_, pend_r_);
        }
        x_ = tr_.challenge_vec(0, current_, pend_l_, pend_r_);  // prover.rs:177-180
        xi_ = fq_inv(x_);
        stage_ = Stage::Vec;
        return kOk;
    }
    const uint32_t L = d_ - (uint32_t)round_, s = 1u << L, h = s / 2;
    if (stage_ == Stage::Vec) {
        if (round_ == 0 && cached_.entry) {
            // round 0's vector stage was the last reader of the cached family
            ctx_->prover_cache()->release(cached_);
            cached_ = ProverGenCache::Ref{};
        }
        if (fl[0]) return fail(kEInvariant, "vector folding invariant failed");  // prover.rs:204-207
        unpack_module(pinned_, s, ct_);
        unpack_module(pinned_ + slot * 16, h, lp_);
        unpack_module(pinned_ + 2 * slot * 16, h, rp_);
        y_ = tr_.challenge_poly(round_, ct_, lp_, rp_);  // prover.rs:253-259
        yi_ = fq_inv(y_);
        stage_ = Stage::Poly;
        return kOk;
    }
    if (stage_ == Stage::Poly) {
        if (fl[1]) return fail(kEInvariant, "round folding invariant failed");  // prover.rs:288-291
        RoundRecord rec;
        rec.round = round_;
        rec.l_vec = std::move(pend_l_);
        rec.r_vec = std::move(pend_r_);
        rec.l_poly = std::move(lp_);
        rec.r_poly = std::move(rp_);
        records_.push_back(std::move(rec));
        unpack_module(pinned_, h, current_);
        if (h >= 2) {
            unpack_module(pinned_ + slot * 16, h, pend_l_);
            unpack_module(pinned_ + 2 * slot * 16, h, pend_r_);
        } else {
            pend_l_ = Module::zero(h);
            pend_r_ = Module::zero(h);
        }
        N_ = n_ = h;
        round_ += 1;
        if (round_ == d_) {
            const uint4* m = reinterpret_cast<const uint4*>(tail + 48);
            opening_ = fq{{m->x, m->y, m->z, m->w}};
            have_opening_ = true;
            stage_ = Stage::Done;
            return kOk;
        }
        x_ = tr_.challenge_vec(round_, current_, pend_l_, pend_r_);
        xi_ = fq_inv(x_);
        stage_ = Stage::Vec;
        return kOk;
    }
    return fail(kEState, "no stage to complete");
}

void ProofState::encode_proof(std::vector<uint8_t>* out) const {
    out->clear();
    out->reserve(proof_encoded_size(d_));
    encode_statement(*out, st_);
    put_u64(*out, records_.size());
    for (const auto& r : records_) encode_record(*out, r);
    const size_t base = out->size();
    out->resize(base + 16);
    fq_to_bytes(opening_, out->data() + base);
}

// ============================================================== GpuProver

GpuProver::~GpuProver() {
    if (s_) cudaStreamSynchronize(s_);
    ps_.release();  // stream-ordered frees on s_, before the stream goes away
    if (s_) {
        cudaStreamSynchronize(s_);
        cudaStreamDestroy(s_);
    }
    if (ev_start_) cudaEventDestroy(ev_start_);
    if (ev_end_) cudaEventDestroy(ev_end_);
}

int GpuProver::fail(int code, const std::string& msg) {
    failed_ = true;
    ctx_->set_error(msg);
    return code;
}

int GpuProver::init(const uint8_t* file, uint64_t len, bool on_device, const uint8_t seed[32], const uint8_t epoch[32],
                    uint64_t max_preprocess_bytes) {
    cudaError_t e = cudaSetDevice(ctx_->device());
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&ev_start_);
    if (e == cudaSuccess) e = cudaEventCreate(&ev_end_);
    if (e != cudaSuccess) return fail(kECuda, std::string("stream/event setup: ") + cudaGetErrorString(e));
    cudaEventRecord(ev_start_, s_);
    int rc = ps_.setup(file, len, on_device, seed, epoch, max_preprocess_bytes, s_);
    if (rc != kOk) return fail(rc, ps_.error());
    return run_stage();  // Init: commitment and round 0's vector cross terms
}

int GpuProver::run_stage() {
    NvtxRange range(stage_name((int)ps_.stage()));
    Plan plan;
    ps_.plan_stage(plan);
    std::string err;
    const int n = plan.launch(ctx_, s_, &err);
    if (n < 0) return fail(kECuda, err);
    const bool last = ps_.stage() == Stage::Poly && ps_.round() + 1 == ps_.depth();
    if (last) cudaEventRecord(ev_end_, s_);
    cudaError_t e = cudaStreamSynchronize(s_);
    if (e != cudaSuccess) return fail(kECuda, std::string("stage: ") + cudaGetErrorString(e));
    int rc;
    {
        NvtxRange fs("fiat-shamir");
        rc = ps_.complete_stage();
    }
    if (rc != kOk) return fail(rc, ps_.error());
    return kOk;
}

int GpuProver::fold_round(uint64_t j, RoundRecord* out, double times_ms[3]) {
    if (failed_) return fail(kEState, "prover is in a failed state");
    if (j != ps_.round()) return fail(kEState, "round index mismatch");
    if (ps_.stage() != Stage::Vec) return fail(kEState, "all rounds have finished");
    using Clk = std::chrono::steady_clock;
    const Clk::time_point t0 = Clk::now();
    int rc = run_stage();  // vector stage
    if (rc != kOk) return rc;
    const Clk::time_point t1 = Clk::now();
    rc = run_stage();  // poly stage
    if (rc != kOk) return rc;
    const Clk::time_point t2 = Clk::now();
    if (out) *out = ps_.records().back();
    if (times_ms) {
        times_ms[0] = std::chrono::duration<double, std::milli>(t1 - t0).count();
        times_ms[1] = std::chrono::duration<double, std::milli>(t2 - t1).count();
        times_ms[2] = std::chrono::duration<double, std::milli>(t2 - t0).count();
    }
    return kOk;
}

double GpuProver::device_ms() const {
    float ms = 0.f;
    if (!ev_start_ || !ev_end_ || cudaEventElapsedTime(&ms, ev_start_, ev_end_) != cudaSuccess) return -1.0;
    return ms;
}

int prove_all(Context* ctx, const uint8_t* file, uint64_t len, bool on_device, const uint8_t seed[32],
              const uint8_t epoch[32], std::vector<uint8_t>* proof, double* device_ms) {
    GpuProver p(ctx);
    int rc = p.init(file, len, on_device, seed, epoch, ctx->max_preprocess());
    if (rc != kOk) return rc;
    for (uint32_t r = 0; r < p.rounds_total(); ++r) {
        rc = p.fold_round(r, nullptr);
        if (rc != kOk) return rc;
    }
    fq o;
    if (!p.final_opening(&o)) {
        ctx->set_error("final opening unavailable");
        return kEState;
    }
    p.encode_proof(proof);
    if (device_ms) *device_ms = p.device_ms();
    return kOk;
}

}  // namespace dm
