/* Prototype-only stand-in: the reference includes this header but calls nothing from it. */
#ifndef CUSPX_SHIM_OPENSSL_CONF_H
#define CUSPX_SHIM_OPENSSL_CONF_H
#endif
