/*
 * cuspx_rng.h -- the NIST AES-256 CTR DRBG behind the drop-in API.
 *
 * Replaces the reference's rng.h interface (rng.h:48-55, rng.cu:139-186):
 *   randombytes_init(entropy, personalization, strength) -> cuspx_randombytes_init
 *   randombytes(x, xlen)                                  -> cuspx_randombytes
 * Same DRBG construction and output stream; AES-256 is built in (no OpenSSL).
 *
 * cuspx_set_deterministic mirrors the reference's unconditional DEBUG_MODE
 * (all_option.h:75), which is ON as shipped: crypto_sign_keypair still draws
 * 3n DRBG bytes but uses the seed 0..3n-1 (sign.cu:344-349), and
 * crypto_sign_signature draws n bytes but uses optrand = 0xAD * n
 * (sign.cu:1950-1954).  Default: on (1), as shipped.
 */
#ifndef CUSPX_RNG_H
#define CUSPX_RNG_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
void cuspx_randombytes_init(const uint8_t entropy[48], const uint8_t *personalization, int security_strength);
int cuspx_randombytes(uint8_t *x, unsigned long long xlen);
void cuspx_aes256_ecb(const uint8_t key[32], const uint8_t in[16], uint8_t out[16]);
void cuspx_set_deterministic(int on);
int cuspx_deterministic(void);
#ifdef __cplusplus
}
#endif
#endif
