/*
 * spx_api.h -- NIST signature API, the drop-in replacement for the
 * reference's api.h (api.h:19-136) and rng.h (rng.h:48-55).
 *
 * One shared library per parameter set, libspx_<set>.so (for example
 * libspx_sha256-128f-simple.so), exports exactly these names with the
 * reference's semantics; the work runs on the GPU through libcuspx.so.
 * The set is fixed when the library is built, as the reference fixes it
 * with -D flags (Makefile:109-155).
 *
 * Conventions (sign.cu:3048-3121, :6058-6079):
 *   - return 0 on success; verify/open return -1 on any failure;
 *   - crypto_sign_open zero-fills m over smlen bytes and sets *mlen = 0 on
 *     failure; sm = sig || m; in-place open (m == sm) is allowed;
 *   - crypto_sign_keypair draws 3n bytes and crypto_sign_signature n bytes
 *     from the process-global DRBG, in that order, like the reference.
 * Unlike the reference these calls are thread-safe.
 */
#ifndef SPX_API_H
#define SPX_API_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
#define CRYPTO_ALGNAME "SPHINCS+"

/* sign.cu:124-147 */
unsigned long long crypto_sign_secretkeybytes(void);
unsigned long long crypto_sign_publickeybytes(void);
unsigned long long crypto_sign_bytes(void);
unsigned long long crypto_sign_seedbytes(void);

/* sign.cu:154 -- sk = SK_SEED || SK_PRF || PUB_SEED || ROOT, pk = PUB_SEED || ROOT */
int crypto_sign_seed_keypair(unsigned char *pk, unsigned char *sk, const unsigned char *seed);
/* sign.cu:342 */
int crypto_sign_keypair(unsigned char *pk, unsigned char *sk);
/* sign.cu:1924 */
int crypto_sign_signature(uint8_t *sig, size_t *siglen, const uint8_t *m, size_t mlen, const uint8_t *sk);
/* sign.cu:3048 */
int crypto_sign_verify(const uint8_t *sig, size_t siglen, const uint8_t *m, size_t mlen, const uint8_t *pk);
/* sign.cu:3302 */
int crypto_sign(unsigned char *sm, unsigned long long *smlen, const unsigned char *m, unsigned long long mlen,
                const unsigned char *sk);
/* sign.cu:6058 */
int crypto_sign_open(unsigned char *m, unsigned long long *mlen, const unsigned char *sm, unsigned long long smlen,
                     const unsigned char *pk);

/* rng.h:48-55 */
void randombytes_init(unsigned char *entropy_input, unsigned char *personalization_string, int security_strength);
int randombytes(unsigned char *x, unsigned long long xlen);

#ifdef __cplusplus
}
#endif
#endif
