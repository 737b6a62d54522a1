// drbg.cpp -- NIST AES-256 CTR DRBG for the drop-in API's randombytes.
//
// Same construction and byte stream as the reference rng.cu:139-241
// (randombytes_init / randombytes / AES256_CTR_DRBG_Update), which calls
// OpenSSL's AES-256-ECB; here AES-256 is implemented directly from FIPS 197
// so the library has no OpenSSL dependency.  State is process-global like
// the reference's DRBG_ctx and guarded by a mutex.
#include <stdint.h>
#include <string.h>

#include <mutex>

#include "../../include/cuspx_rng.h"

namespace {

struct Aes256 {
    uint8_t rk[240];
    static uint8_t sbox(uint8_t x) {
        static uint8_t tab[256];
        static bool ready = false;
        static std::once_flag once;
        std::call_once(once, [] {
            // S-box: inverse in GF(2^8) mod x^8+x^4+x^3+x+1, then the FIPS 197 affine map
            uint8_t p = 1, q = 1;
            do {
                p = (uint8_t)(p ^ (p << 1) ^ ((p & 0x80) ? 0x1b : 0));  // p *= 3
                q ^= q << 1; q ^= q << 2; q ^= q << 4;                   // q /= 3
                if (q & 0x80) q ^= 0x09;
                uint8_t s = q ^ (uint8_t)((q << 1) | (q >> 7)) ^ (uint8_t)((q << 2) | (q >> 6)) ^
                            (uint8_t)((q << 3) | (q >> 5)) ^ (uint8_t)((q << 4) | (q >> 4));
                tab[p] = s ^ 0x63;
            } while (p != 1);
            tab[0] = 0x63;
            ready = true;
        });
        (void)ready;
        return tab[x];
    }
    static uint8_t xt(uint8_t a) { return (uint8_t)((a << 1) ^ ((a & 0x80) ? 0x1b : 0)); }

    explicit Aes256(const uint8_t key[32]) {
        memcpy(rk, key, 32);
        uint8_t rcon = 1;
        for (int i = 8; i < 60; i++) {
            uint8_t t[4];
            memcpy(t, rk + 4 * (i - 1), 4);
            if (i % 8 == 0) {
                const uint8_t u = t[0];
                t[0] = sbox(t[1]) ^ rcon;
                t[1] = sbox(t[2]);
                t[2] = sbox(t[3]);
                t[3] = sbox(u);
                rcon = xt(rcon);
            } else if (i % 8 == 4) {
                for (auto &b : t) b = sbox(b);
            }
            for (int j = 0; j < 4; j++) rk[4 * i + j] = rk[4 * (i - 8) + j] ^ t[j];
        }
    }
    void encrypt(const uint8_t in[16], uint8_t out[16]) const {
        uint8_t s[16];
        for (int i = 0; i < 16; i++) s[i] = in[i] ^ rk[i];
        for (int r = 1; r <= 14; r++) {
            uint8_t t[16];
            // SubBytes + ShiftRows (state is column-major: byte 4c+row)
            for (int c = 0; c < 4; c++)
                for (int row = 0; row < 4; row++) t[4 * c + row] = sbox(s[4 * ((c + row) & 3) + row]);
            if (r < 14) {
                for (int c = 0; c < 4; c++) {
                    const uint8_t a0 = t[4 * c], a1 = t[4 * c + 1], a2 = t[4 * c + 2], a3 = t[4 * c + 3];
                    const uint8_t all = a0 ^ a1 ^ a2 ^ a3;
                    s[4 * c] = a0 ^ all ^ xt(a0 ^ a1);
                    s[4 * c + 1] = a1 ^ all ^ xt(a1 ^ a2);
                    s[4 * c + 2] = a2 ^ all ^ xt(a2 ^ a3);
                    s[4 * c + 3] = a3 ^ all ^ xt(a3 ^ a0);
                }
            } else {
                memcpy(s, t, 16);
            }
            for (int i = 0; i < 16; i++) s[i] ^= rk[16 * r + i];
        }
        memcpy(out, s, 16);
    }
};

struct Drbg {
    uint8_t key[32] = {0};
    uint8_t v[16] = {0};
    int reseed = 0;
    static void inc(uint8_t v[16]) {
        for (int j = 15; j >= 0; j--) {
            if (v[j] == 0xff) v[j] = 0;
            else { v[j]++; break; }
        }
    }
    void update(const uint8_t *provided) {
        uint8_t tmp[48];
        Aes256 aes(key);
        for (int i = 0; i < 3; i++) {
            inc(v);
            aes.encrypt(v, tmp + 16 * i);
        }
        if (provided)
            for (int i = 0; i < 48; i++) tmp[i] ^= provided[i];
        memcpy(key, tmp, 32);
        memcpy(v, tmp + 32, 16);
    }
};

Drbg g_drbg;
std::mutex g_mu;
int g_deterministic = 1;

}  // namespace

extern "C" {

void cuspx_randombytes_init(const uint8_t entropy[48], const uint8_t *personalization, int security_strength) {
    (void)security_strength;
    std::lock_guard<std::mutex> lk(g_mu);
    uint8_t seed[48];
    memcpy(seed, entropy, 48);
    if (personalization)
        for (int i = 0; i < 48; i++) seed[i] ^= personalization[i];
    memset(g_drbg.key, 0, 32);
    memset(g_drbg.v, 0, 16);
    g_drbg.update(seed);
    g_drbg.reseed = 1;
}

int cuspx_randombytes(uint8_t *x, unsigned long long xlen) {
    std::lock_guard<std::mutex> lk(g_mu);
    uint8_t blk[16];
    Aes256 aes(g_drbg.key);
    while (xlen > 0) {
        Drbg::inc(g_drbg.v);
        aes.encrypt(g_drbg.v, blk);
        const size_t take = xlen > 15 ? 16 : (size_t)xlen;
        memcpy(x, blk, take);
        x += take;
        xlen -= take;
    }
    g_drbg.update(nullptr);
    g_drbg.reseed++;
    return 0;
}

void cuspx_aes256_ecb(const uint8_t key[32], const uint8_t in[16], uint8_t out[16]) {
    Aes256 aes(key);
    aes.encrypt(in, out);
}

void cuspx_set_deterministic(int on) { g_deterministic = on ? 1 : 0; }
int cuspx_deterministic(void) { return g_deterministic; }

}  // extern "C"
