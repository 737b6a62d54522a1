/* Prototype-only stand-in: the one libcrypto error routine the reference DRBG names. */
#ifndef CUSPX_SHIM_OPENSSL_ERR_H
#define CUSPX_SHIM_OPENSSL_ERR_H
#include <stdio.h>
#ifdef __cplusplus
extern "C" {
#endif
void ERR_print_errors_fp(FILE *fp);
#ifdef __cplusplus
}
#endif
#endif
