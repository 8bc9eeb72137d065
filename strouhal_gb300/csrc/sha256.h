// SHA-256 (FIPS 180-4), streaming interface. Used for the state digest.
#pragma once

#include <cstddef>
#include <cstdint>

namespace stro {

struct Sha256 {
    uint32_t h[8];
    uint8_t buf[64];
    uint64_t total = 0;
    size_t fill = 0;
    Sha256();
    void update(const void* data, size_t len);
    void finish(uint8_t out[32]);
};

void sha256_hex(const uint8_t digest[32], char hex[65]);

}  // namespace stro
