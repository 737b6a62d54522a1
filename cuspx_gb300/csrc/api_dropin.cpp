// api_dropin.cpp -- the NIST api.h names for one parameter set, built once
// per set as libspx_<set>.so with -DCUSPX_SET_NAME="<set>".  Each call is a
// one-item batch on the GPU (the plain one-signature-per-call path).
//
// Semantics follow the reference CPU API: sign.cu:124-182 (sizes, keypair),
// :342-353 (crypto_sign_keypair), :1924-1994 (crypto_sign_signature),
// :3048-3121 (crypto_sign_verify), :3302-3311 (crypto_sign),
// :6058-6079 (crypto_sign_open).
#include <stdlib.h>
#include <string.h>

#include <mutex>
#include <vector>

#include "../../include/cuspx.h"
#include "../../include/cuspx_rng.h"
#include "../../include/spx_api.h"

#ifndef CUSPX_SET_NAME
#error "build with -DCUSPX_SET_NAME=\"sha256-128f-simple\" (or another set)"
#endif

namespace {
std::once_flag g_sizes_once, g_ctx_once;
cuspx_ctx *g_ctx = nullptr;
int g_set = -1;
size_t g_pk, g_sk, g_sig, g_seed;
int g_n;

// sizes need no GPU
void sizes() {
    std::call_once(g_sizes_once, [] {
        g_set = cuspx_set_id(CUSPX_SET_NAME);
        cuspx_set_sizes(g_set, &g_pk, &g_sk, &g_sig, &g_seed, &g_n);
    });
}

// the process-wide context on device $CUSPX_DEVICE (default 0)
bool ready() {
    sizes();
    std::call_once(g_ctx_once, [] {
        const char *dev = getenv("CUSPX_DEVICE");
        if (cuspx_create(dev ? atoi(dev) : 0, &g_ctx) != CUSPX_OK) g_ctx = nullptr;
    });
    return g_ctx != nullptr;
}
}  // namespace

extern "C" {

unsigned long long crypto_sign_secretkeybytes(void) { sizes(); return g_sk; }
unsigned long long crypto_sign_publickeybytes(void) { sizes(); return g_pk; }
unsigned long long crypto_sign_bytes(void) { sizes(); return g_sig; }
unsigned long long crypto_sign_seedbytes(void) { sizes(); return g_seed; }

int crypto_sign_seed_keypair(unsigned char *pk, unsigned char *sk, const unsigned char *seed) {
    if (!ready()) return -1;
    return cuspx_keypair_batch(g_ctx, g_set, 1, seed, pk, sk) == CUSPX_OK ? 0 : -1;
}

int crypto_sign_keypair(unsigned char *pk, unsigned char *sk) {
    if (!ready()) return -1;
    unsigned char seed[96];
    cuspx_randombytes(seed, g_seed);
    if (cuspx_deterministic())
        for (size_t i = 0; i < g_seed; i++) seed[i] = (unsigned char)i;
    return crypto_sign_seed_keypair(pk, sk, seed);
}

int crypto_sign_signature(uint8_t *sig, size_t *siglen, const uint8_t *m, size_t mlen, const uint8_t *sk) {
    if (!ready()) return -1;
    uint8_t optrand[32];
    cuspx_randombytes(optrand, g_n);
    if (cuspx_deterministic()) memset(optrand, 0xad, g_n);
    const uint64_t off = 0, len = mlen;
    int32_t st = 0;
    int rc = cuspx_sign_batch(g_ctx, g_set, 1, sk, m, &off, &len, optrand, sig, &st);
    if (rc != CUSPX_OK) return -1;
    if (siglen) *siglen = g_sig;
    return 0;
}

int crypto_sign_verify(const uint8_t *sig, size_t siglen, const uint8_t *m, size_t mlen, const uint8_t *pk) {
    if (!ready()) return -1;
    if (siglen != g_sig) return -1;
    const uint64_t off = 0, len = mlen;
    int32_t verdict = -1;
    if (cuspx_verify_batch(g_ctx, g_set, 1, pk, m, &off, &len, sig, nullptr, &verdict) != CUSPX_OK) return -1;
    return verdict == 0 ? 0 : -1;
}

int crypto_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m, unsigned long long mlen,
                const unsigned char *sk) {
    sizes();
    // m may alias sm + sig bytes (in-place signing); sign from a copy
    std::vector<unsigned char> mc(m, m + mlen);
    size_t siglen = 0;
    if (crypto_sign_signature(sm, &siglen, mc.data(), (size_t)mlen, sk)) return -1;
    memmove(sm + g_sig, mc.data(), mlen);
    *smlen = siglen + mlen;
    return 0;
}

int crypto_sign_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm, unsigned long long smlen,
                     const unsigned char *pk) {
    sizes();
    if (smlen < g_sig) {
        memset(m, 0, smlen);
        *mlen = 0;
        return -1;
    }
    *mlen = smlen - g_sig;
    if (crypto_sign_verify(sm, g_sig, sm + g_sig, (size_t)*mlen, pk)) {
        memset(m, 0, smlen);
        *mlen = 0;
        return -1;
    }
    memmove(m, sm + g_sig, *mlen);
    return 0;
}

// ---- the reference's GPU faces -------------------------------------------

static int batch_keypair(unsigned char *pk, unsigned char *sk, unsigned int num) {
    if (!ready()) return -1;
    std::vector<unsigned char> seeds((size_t)num * g_seed);
    for (unsigned int i = 0; i < num; i++) {
        unsigned char *sd = seeds.data() + (size_t)i * g_seed;
        cuspx_randombytes(sd, g_seed);
        if (cuspx_deterministic())
            for (size_t j = 0; j < g_seed; j++) sd[j] = (unsigned char)j;
    }
    return cuspx_keypair_batch(g_ctx, g_set, num, seeds.data(), pk, sk) == CUSPX_OK ? 0 : -1;
}

// num messages of mlen bytes -> num rows of sig || m_i
static int batch_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m, unsigned long long mlen,
                      const unsigned char *sk, unsigned int num) {
    if (!ready()) return -1;
    if (num == 0) return 0;
    std::vector<uint64_t> off(num), len(num, mlen);
    for (unsigned int i = 0; i < num; i++) off[i] = (uint64_t)i * mlen;
    std::vector<unsigned char> opt((size_t)num * g_n), sigs((size_t)num * g_sig);
    for (unsigned int i = 0; i < num; i++) {
        cuspx_randombytes(opt.data() + (size_t)i * g_n, g_n);
        if (cuspx_deterministic()) memset(opt.data() + (size_t)i * g_n, 0xad, g_n);
    }
    std::vector<int32_t> st(num);
    std::vector<unsigned char> mc(m, m + (size_t)num * mlen);   // m may alias sm
    if (cuspx_sign_batch(g_ctx, g_set, num, sk, mc.data(), off.data(), len.data(), opt.data(), sigs.data(),
                         st.data()) != CUSPX_OK)
        return -1;
    const size_t row = g_sig + mlen;
    for (unsigned int i = 0; i < num; i++) {
        memcpy(sm + i * row, sigs.data() + (size_t)i * g_sig, g_sig);
        memcpy(sm + i * row + g_sig, mc.data() + (size_t)i * mlen, mlen);
    }
    *smlen = row;
    for (unsigned int i = 0; i < num; i++)
        if (st[i]) return -1;
    return 0;
}

// num rows of smlen bytes (sig || m_i) -> num messages; 0 only if all verify
static int batch_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm, unsigned long long smlen,
                      const unsigned char *pk, unsigned int num) {
    sizes();
    if (num == 0) {
        *mlen = 0;
        return 0;
    }
    if (smlen < g_sig) {
        memset(m, 0, (size_t)num * smlen);
        *mlen = 0;
        return -1;
    }
    if (!ready()) return -1;
    const uint64_t ml = smlen - g_sig;
    std::vector<unsigned char> sigs((size_t)num * g_sig), msgs((size_t)num * ml);
    std::vector<uint64_t> off(num), len(num, ml);
    for (unsigned int i = 0; i < num; i++) {
        memcpy(sigs.data() + (size_t)i * g_sig, sm + i * smlen, g_sig);
        memcpy(msgs.data() + (size_t)i * ml, sm + i * smlen + g_sig, ml);
        off[i] = (uint64_t)i * ml;
    }
    std::vector<int32_t> v(num, -1);
    if (cuspx_verify_batch(g_ctx, g_set, num, pk, msgs.data(), off.data(), len.data(), sigs.data(), nullptr,
                           v.data()) != CUSPX_OK)
        return -1;
    int all = 0;
    for (unsigned int i = 0; i < num; i++) {
        if (v[i] == 0) memcpy(m + i * ml, msgs.data() + (size_t)i * ml, ml);
        else {
            memset(m + i * ml, 0, ml);
            all = -1;
        }
    }
    *mlen = ml;
    return all;
}

int face_crypto_sign_keypair(unsigned char *pk, unsigned char *sk) { return crypto_sign_keypair(pk, sk); }
int face_ap_crypto_sign_keypair(unsigned char *pk, unsigned char *sk) { return crypto_sign_keypair(pk, sk); }
int face_crypto_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m, unsigned long long mlen,
                     const unsigned char *sk) {
    return crypto_sign(sm, smlen, m, mlen, sk);
}
int face_ap_crypto_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m,
                        unsigned long long mlen, const unsigned char *sk) {
    return crypto_sign(sm, smlen, m, mlen, sk);
}
int face_crypto_sign_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm,
                          unsigned long long smlen, const unsigned char *pk) {
    return crypto_sign_open(m, mlen, sm, smlen, pk);
}
int face_ap_crypto_sign_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm,
                             unsigned long long smlen, const unsigned char *pk) {
    return crypto_sign_open(m, mlen, sm, smlen, pk);
}
int face_mdp_crypto_sign_keypair(unsigned char *pk, unsigned char *sk, unsigned int num) {
    return batch_keypair(pk, sk, num);
}
int face_mhp_crypto_sign_keypair(unsigned char *pk, unsigned char *sk, unsigned int num, unsigned int) {
    return batch_keypair(pk, sk, num);
}
int face_mhp_crypto_sign_keypair_scheme2(unsigned char *pk, unsigned char *sk, unsigned int num, unsigned int) {
    return batch_keypair(pk, sk, num);
}
int face_mdp_crypto_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m,
                         unsigned long long mlen, const unsigned char *sk, unsigned int dp_num) {
    return batch_sign(sm, smlen, m, mlen, sk, dp_num);
}
int face_sdp_crypto_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m,
                         unsigned long long mlen, const unsigned char *sk, unsigned int dp_num) {
    return batch_sign(sm, smlen, m, mlen, sk, dp_num);
}
int face_mhp_crypto_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m,
                         unsigned long long mlen, const unsigned char *sk, unsigned int dp_num) {
    return batch_sign(sm, smlen, m, mlen, sk, dp_num);
}
int face_mhp_crypto_sign_scheme2(unsigned char *sm, unsigned long long *smlen, const unsigned char *m,
                                 unsigned long long mlen, const unsigned char *sk, unsigned int dp_num,
                                 unsigned int) {
    return batch_sign(sm, smlen, m, mlen, sk, dp_num);
}
int face_mdp_crypto_sign_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm,
                              unsigned long long smlen, const unsigned char *pk, unsigned int dp_num) {
    return batch_open(m, mlen, sm, smlen, pk, dp_num);
}
int face_sdp_crypto_sign_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm,
                              unsigned long long smlen, const unsigned char *pk, unsigned int dp_num) {
    return batch_open(m, mlen, sm, smlen, pk, dp_num);
}
int face_mhp_crypto_sign_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm,
                              unsigned long long smlen, const unsigned char *pk, unsigned int dp_num,
                              unsigned int) {
    return batch_open(m, mlen, sm, smlen, pk, dp_num);
}

void randombytes_init(unsigned char *entropy_input, unsigned char *personalization_string, int security_strength) {
    cuspx_randombytes_init(entropy_input, personalization_string, security_strength);
}

int randombytes(unsigned char *x, unsigned long long xlen) { return cuspx_randombytes(x, xlen); }

}  // extern "C"
