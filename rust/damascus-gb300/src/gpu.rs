//! Drop-in for `damascus-core`'s `src/utils/gpu.rs`: the same public names and
//! signatures (`cuda_device_info`, `cuda_backend_ready`, `try_fold_pairs_gpu`,
//! `try_ntt_batch_gpu`), backed by this library's implementations of the
//! reference's two CUDA hooks (`damascus_cuda_fold_batch`,
//! `damascus_cuda_ntt_batch`).  The reference's callers
//! (src/protocol/prover.rs:343-362, src/algebra/ntt.rs:157-180) switch by
//! importing this module instead; as there, `None` means "not done on the GPU"
//! and the caller keeps its CPU path for these two helpers.  The protocol-level
//! API of the crate root has no such fallback.
use std::sync::OnceLock;

use crate::sys;

const NTT_BATCH_PRIMES: usize = 8;

#[derive(Clone, Debug)]
pub struct CudaDeviceInfo {
    pub available: bool,
    pub summary: String,
}

static INFO: OnceLock<CudaDeviceInfo> = OnceLock::new();

/// Whether a GB300 context can be created (DAMASCUS_GPU=0 turns the GPU off, as
/// in the reference).  Probed once, by creating and destroying a context.
pub fn cuda_device_info() -> &'static CudaDeviceInfo {
    INFO.get_or_init(|| {
        if std::env::var("DAMASCUS_GPU").is_ok_and(|v| v == "0") {
            return CudaDeviceInfo { available: false, summary: "disabled by DAMASCUS_GPU=0".into() };
        }
        probe()
    })
}

#[cfg(damascus_cuda_available)]
fn probe() -> CudaDeviceInfo {
    match crate::Context::new(0, 1 << 30) {
        Ok(_) => CudaDeviceInfo { available: true, summary: "libdamascus_gb300: sm_103a context on device 0".into() },
        Err(e) => CudaDeviceInfo { available: false, summary: e.to_string() },
    }
}

#[cfg(not(damascus_cuda_available))]
fn probe() -> CudaDeviceInfo {
    CudaDeviceInfo { available: false, summary: "built without libdamascus_gb300".into() }
}

pub fn cuda_backend_ready() -> bool {
    cuda_device_info().available
}

/// out[i] = left[i] + right[i] * challenge mod q (q = 2^112 - 75), over u128 words.
pub fn try_fold_pairs_gpu(left: &[u128], right: &[u128], challenge: u128) -> Option<Vec<u128>> {
    if !cuda_backend_ready() || left.len() != right.len() || left.is_empty() {
        return None;
    }
    #[cfg(damascus_cuda_available)]
    {
        let split = |v: &[u128]| -> (Vec<u64>, Vec<u64>) {
            (v.iter().map(|x| *x as u64).collect(), v.iter().map(|x| (*x >> 64) as u64).collect())
        };
        let (llo, lhi) = split(left);
        let (rlo, rhi) = split(right);
        let n = left.len();
        let (mut olo, mut ohi) = (vec![0u64; n], vec![0u64; n]);
        let rc = unsafe {
            sys::damascus_cuda_fold_batch(llo.as_ptr(), lhi.as_ptr(), rlo.as_ptr(), rhi.as_ptr(), olo.as_mut_ptr(),
                                          ohi.as_mut_ptr(), n, challenge as u64, (challenge >> 64) as u64)
        };
        if rc != 0 {
            return None;
        }
        Some(olo.iter().zip(ohi.iter()).map(|(&lo, &hi)| lo as u128 | (hi as u128) << 64).collect())
    }
    #[cfg(not(damascus_cuda_available))]
    {
        let _ = challenge;
        None
    }
}

/// For each of the eight CRT primes, the length-n cyclic convolution of a[p] and
/// b[p] (residues below the prime).  The root tables are checked for shape only,
/// as the library derives its own.
pub fn try_ntt_batch_gpu(a: &[Vec<u64>], b: &[Vec<u64>], n: usize, primes: &[u64; NTT_BATCH_PRIMES],
                         stage_roots: &[u64], inv_roots: &[u64], inv_sizes: &[u64; NTT_BATCH_PRIMES])
                         -> Option<Vec<Vec<u64>>> {
    if !cuda_backend_ready() || n == 0 || !n.is_power_of_two() || a.len() != NTT_BATCH_PRIMES
        || b.len() != NTT_BATCH_PRIMES {
        return None;
    }
    let log_n = n.trailing_zeros() as usize;
    if stage_roots.len() != NTT_BATCH_PRIMES * log_n || inv_roots.len() != NTT_BATCH_PRIMES * log_n
        || a.iter().chain(b.iter()).any(|v| v.len() != n) {
        return None;
    }
    #[cfg(damascus_cuda_available)]
    {
        let flat_a: Vec<u64> = a.iter().flatten().copied().collect();
        let flat_b: Vec<u64> = b.iter().flatten().copied().collect();
        let mut out = vec![0u64; NTT_BATCH_PRIMES * n];
        let rc = unsafe {
            sys::damascus_cuda_ntt_batch(flat_a.as_ptr(), flat_b.as_ptr(), out.as_mut_ptr(), n, primes.as_ptr(),
                                         stage_roots.as_ptr(), inv_roots.as_ptr(), inv_sizes.as_ptr())
        };
        if rc != 0 {
            return None;
        }
        Some(out.chunks_exact(n).map(|c| c.to_vec()).collect())
    }
    #[cfg(not(damascus_cuda_available))]
    {
        let _ = (primes, inv_sizes);
        None
    }
}
