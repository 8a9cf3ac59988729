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
}  // namespace kc
