// pa_sha3.cpp -- SHA3-256 (FIPS 202): Keccak-f[1600] sponge, rate 136 bytes, domain bits 01 + pad10*1.
// The round constants and rotation offsets are generated from the standard's definitions (the rc(t)
// LFSR and the (x, y) -> (y, 2x + 3y) walk) rather than tabled.
#include "../../include/pa_service.h"

#include <cstring>

namespace {

struct KeccakTables {
    uint64_t rc[24];
    int rot[25];  // rot[x + 5y]
    KeccakTables() {
        // rc(t): LFSR x^8 + x^6 + x^5 + x^4 + 1 over GF(2), state starts at 1
        auto rc_bit = [](int t) {
            if (t % 255 == 0) return 1u;
            unsigned r = 1;
            for (int i = 1; i <= t % 255; ++i) {
                r <<= 1;
                if (r & 0x100) r ^= 0x171;
            }
            return r & 1u;
        };
        for (int ir = 0; ir < 24; ++ir) {
            uint64_t c = 0;
            for (int j = 0; j <= 6; ++j)
                if (rc_bit(j + 7 * ir)) c |= 1ull << ((1 << j) - 1);
            rc[ir] = c;
        }
        rot[0] = 0;
        int x = 1, y = 0;
        for (int t = 0; t < 24; ++t) {
            rot[x + 5 * y] = ((t + 1) * (t + 2) / 2) % 64;
            int nx = y, ny = (2 * x + 3 * y) % 5;
            x = nx;
            y = ny;
        }
    }
};

const KeccakTables& tables() {
    static const KeccakTables t;
    return t;
}

inline uint64_t rotl(uint64_t v, int r) { return r ? (v << r) | (v >> (64 - r)) : v; }

void keccak_f(uint64_t a[25]) {
    const KeccakTables& T = tables();
    for (int ir = 0; ir < 24; ++ir) {
        uint64_t c[5], d[5], b[25];
        for (int x = 0; x < 5; ++x) c[x] = a[x] ^ a[x + 5] ^ a[x + 10] ^ a[x + 15] ^ a[x + 20];
        for (int x = 0; x < 5; ++x) d[x] = c[(x + 4) % 5] ^ rotl(c[(x + 1) % 5], 1);
        for (int i = 0; i < 25; ++i) a[i] ^= d[i % 5];
        // rho and pi: B[y, 2x + 3y] = rot(A[x, y], r[x, y])
        for (int x = 0; x < 5; ++x)
            for (int y = 0; y < 5; ++y) b[y + 5 * ((2 * x + 3 * y) % 5)] = rotl(a[x + 5 * y], T.rot[x + 5 * y]);
        // chi
        for (int y = 0; y < 5; ++y)
            for (int x = 0; x < 5; ++x)
                a[x + 5 * y] = b[x + 5 * y] ^ (~b[(x + 1) % 5 + 5 * y] & b[(x + 2) % 5 + 5 * y]);
        a[0] ^= T.rc[ir];  // iota
    }
}

inline uint64_t load_le64(const uint8_t* p) {
    uint64_t v = 0;
    for (int i = 7; i >= 0; --i) v = (v << 8) | p[i];
    return v;
}

}  // namespace

extern "C" void pa_sha3_256(const void* data, size_t len, uint8_t out[32]) {
    constexpr size_t kRate = 136;
    uint64_t a[25] = {};
    const uint8_t* p = static_cast<const uint8_t*>(data);
    while (len >= kRate) {
        for (size_t i = 0; i < kRate / 8; ++i) a[i] ^= load_le64(p + 8 * i);
        keccak_f(a);
        p += kRate;
        len -= kRate;
    }
    uint8_t last[kRate] = {};
    if (len) std::memcpy(last, p, len);
    last[len] ^= 0x06;
    last[kRate - 1] ^= 0x80;
    for (size_t i = 0; i < kRate / 8; ++i) a[i] ^= load_le64(last + 8 * i);
    keccak_f(a);
    for (int i = 0; i < 32; ++i) out[i] = (uint8_t)(a[i / 8] >> (8 * (i % 8)));
}
