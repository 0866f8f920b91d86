// Host-only: prints the tcgen05 instruction and shared-memory descriptors that umma.cuh encodes,
// for the CPU test of their bit fields (no device code runs).
#include <cinttypes>
#include <cstdio>

#include "umma.cuh"

int main() {
    const int shapes[][2] = {{128, 48}, {128, 96}, {128, 192}, {128, 16}, {128, 256}, {64, 8}};
    for (const auto& s : shapes) printf("idesc %d %d %u\n", s[0], s[1], gbc::umma::idesc_bf16_f32(s[0], s[1]));
    const unsigned addrs[] = {0u, 1024u, 0x8000u + 32u, 0x38000u + 96u, 227u * 1024u};
    for (unsigned a : addrs) printf("sdesc %u %" PRIu64 "\n", a, (uint64_t)gbc::umma::sdesc_sw128(a));
    return 0;
}
