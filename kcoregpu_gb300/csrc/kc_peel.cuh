// Launch shape of the persistent single-graph peel.
#pragma once
#include "kc_device.cuh"

namespace kc {
constexpr int kPeelThreads = 512;
constexpr int kPeelWarps = kPeelThreads / 32;
const void* peel_persistent_fn();
// Same kernel with every global and shared index bounds-checked (violations are
// recorded in PeelCtl and skipped); selected with KC_CHECKED=1 in the environment.
const void* peel_persistent_fn_checked();
// The persistent kernel the single-graph entry points launch: the
// bounds-checked one when KC_CHECKED=1 is set in the environment.
const void* peel_kernel_selected();
// Time limit (us) of the single-graph peel's device waits (2 s; KC_WAIT_US
// shortens it for the tests that make a wait run out).
uint32_t wait_limit_us();
// One-CTA tail peel (kTailThreads threads, peel_tail_smem() bytes of dynamic
// shared memory), launched after the persistent kernel on the same stream.
const void* peel_tail_fn();
size_t peel_tail_smem();
// Cluster h-index tail (kc_hxtail.cu): one cluster of peel_hxtail_cluster()
// CTAs of peel_hxtail_threads() threads and peel_hxtail_smem() bytes of
// dynamic shared memory, launched after the persistent kernel and before the
// level tail kernel.
const void* peel_hxtail_fn();
size_t peel_hxtail_smem();
int peel_hxtail_cluster();
int peel_hxtail_threads();
// h-index peel (kc_hindex.cu): one cooperative launch of kPeelThreads-thread
// CTAs, one per SM, launched before the persistent kernel, which returns at
// once when it set HxCtl::solved.
const void* peel_hindex_fn();
// Device-side CSR validation (kc_validate.cu), stream-ordered before a peel
// launched with max_level = 0xFFFFFFFF; returns 0 or -1 (launch error).
int launch_validate_csr(const uint32_t* off, const uint32_t* nbr, uint32_t V, uint64_t E, PeelCtl* ctl,
                        cudaStream_t stream);
}  // namespace kc
