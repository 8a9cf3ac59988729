// Launch shape of the persistent single-graph peel.
#pragma once
#include "kc_device.cuh"

namespace kc {
constexpr int kPeelThreads = 512;
constexpr int kPeelWarps = kPeelThreads / 32;
const void* peel_persistent_fn();
}  // namespace kc
