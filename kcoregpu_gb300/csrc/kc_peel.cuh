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
// One-CTA tail peel (kTailThreads threads, peel_tail_smem() bytes of dynamic
// shared memory), launched after the persistent kernel on the same stream.
const void* peel_tail_fn();
size_t peel_tail_smem();
}  // namespace kc
