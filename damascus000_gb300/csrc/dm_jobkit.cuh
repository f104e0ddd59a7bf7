// Device-side helpers shared by the multi-job kernels: a job list passed by
// value in kernel parameters, the job of the current block, 16-byte Z_q loads.
#pragma once

#include <cuda_runtime.h>

#include "dm_jobs.cuh"

namespace dm {
namespace jobkit {

template <class J>
struct JobList {
    J j[kMaxJobs];
    int n;
};

// Job of this block (jobs are sorted by cta0; at most kMaxJobs, uniform per block).
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

// Numbers the blocks of each job consecutively and copies the jobs into L.
template <class J>
inline uint32_t assign_ctas(J* jobs, int n, JobList<J>& L, uint64_t (*ctas_of)(const J&)) {
    uint64_t total = 0;
    L.n = n;
    for (int i = 0; i < n; ++i) {
        jobs[i].cta0 = (uint32_t)total;
        L.j[i] = jobs[i];
        total += ctas_of(jobs[i]);
    }
    return (uint32_t)total;
}

}  // namespace jobkit
}  // namespace dm
