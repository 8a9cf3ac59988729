// Internal helpers shared by the host translation units of libkcore_gb300.
#pragma once
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>
#include "kcore.h"

namespace kc {

// Thread-local message for the last error (kc_last_error()).
void set_error_msg(const std::string& msg);

// Counter-based generator: splitmix64 finaliser over (seed, stream, counter).
// Deterministic on any host and independent of the thread count.
static inline uint64_t mix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
static inline uint64_t rnd(uint64_t seed, uint64_t stream, uint64_t ctr) {
    return mix64(mix64(seed ^ 0xD1B54A32D192ED03ull) ^ mix64(stream * 0x9E3779B97F4A7C15ull + ctr));
}
static inline double rnd_unit(uint64_t seed, uint64_t stream, uint64_t ctr) {
    return (double)(rnd(seed, stream, ctr) >> 11) * (1.0 / 9007199254740992.0);
}

// Builds the reference CSR (graph.cpp:84-122 semantics) from raw directed
// edges; self-loops are expected to be already dropped when `loops_dropped`.
int build_csr(const uint32_t* src, const uint32_t* dst, uint64_t n, kc_csr_host* out);

// Seeded Fisher-Yates permutation of [0, n).
void seeded_permutation(uint32_t n, uint64_t seed, std::vector<uint32_t>& perm);

}  // namespace kc
