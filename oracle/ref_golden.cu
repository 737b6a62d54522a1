// Line-oriented driver over the reference's own CPU SPHINCS+ implementation.
//
// Test infrastructure only: it is compiled by oracle/build_ref.sh together
// with the reference sources (sign.cu, wots.cu, fors.cu, utils.cu, sha256.cu,
// fips202.cu, hash_*.cu, thash_*.cu, address.cu, rng.cu, common.cu) exactly
// where they lie, for one parameter set per build, and is used to pin the C
// restatement in oracle/spx_oracle.c and to write tests/golden fixtures.
//
// Protocol: one command per stdin line, one answer per stdout line, hex
// encoded.  Commands mirror the reference api.h / rng.h entry points:
//   info                         -> "n pkbytes skbytes sigbytes seedbytes"
//   drbg_init <entropy48>        -> randombytes_init (rng.cu:139)
//   drbg <len>                   -> randombytes (rng.cu:155)
//   seedkp <seed3n>              -> crypto_sign_seed_keypair (sign.cu:154): "<pk> <sk>"
//   kp                           -> crypto_sign_keypair (sign.cu:342): "<pk> <sk>"
//   sign <sk> <msg|->            -> crypto_sign_signature (sign.cu:1924): "<sig>"
//   verify <pk> <sig> <msg|->    -> crypto_sign_verify (sign.cu:3048): "<rc>"
//   smsign <sk> <msg|->          -> crypto_sign (sign.cu:3302): "<sm>"
//   open <pk> <sm>               -> crypto_sign_open (sign.cu:6058): "<rc> <mlen> <m|->"
//   time_sign <sk> <mlen> <reps> -> seconds per crypto_sign_signature call
// An empty byte string is written as "-".
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "api.h"
#include "rng.h"

static std::vector<unsigned char> unhex(const std::string &s) {
    std::vector<unsigned char> out;
    if (s == "-") return out;
    out.resize(s.size() / 2);
    for (size_t i = 0; i < out.size(); i++) out[i] = (unsigned char)strtoul(s.substr(2 * i, 2).c_str(), nullptr, 16);
    return out;
}

static std::string hex(const unsigned char *p, size_t n) {
    static const char *d = "0123456789abcdef";
    if (n == 0) return "-";
    std::string s(2 * n, '0');
    for (size_t i = 0; i < n; i++) { s[2 * i] = d[p[i] >> 4]; s[2 * i + 1] = d[p[i] & 15]; }
    return s;
}

int main() {
    std::ios::sync_with_stdio(false);
    const size_t PK = crypto_sign_publickeybytes(), SK = crypto_sign_secretkeybytes();
    const size_t SIG = crypto_sign_bytes(), SEED = crypto_sign_seedbytes();
    std::string line;
    while (std::getline(std::cin, line)) {
        std::istringstream in(line);
        std::string cmd;
        in >> cmd;
        if (cmd == "info") {
            std::cout << SPX_N << " " << PK << " " << SK << " " << SIG << " " << SEED << "\n";
        } else if (cmd == "drbg_init") {
            std::string e; in >> e;
            auto ent = unhex(e);
            randombytes_init(ent.data(), nullptr, 256);
            std::cout << "ok\n";
        } else if (cmd == "drbg") {
            unsigned long long n; in >> n;
            std::vector<unsigned char> b(n + 1);
            randombytes(b.data(), n);
            std::cout << hex(b.data(), n) << "\n";
        } else if (cmd == "seedkp") {
            std::string s; in >> s;
            auto seed = unhex(s);
            std::vector<unsigned char> pk(PK), sk(SK);
            crypto_sign_seed_keypair(pk.data(), sk.data(), seed.data());
            std::cout << hex(pk.data(), PK) << " " << hex(sk.data(), SK) << "\n";
        } else if (cmd == "kp") {
            std::vector<unsigned char> pk(PK), sk(SK);
            crypto_sign_keypair(pk.data(), sk.data());
            std::cout << hex(pk.data(), PK) << " " << hex(sk.data(), SK) << "\n";
        } else if (cmd == "sign") {
            std::string a, b; in >> a >> b;
            auto sk = unhex(a); auto m = unhex(b);
            m.reserve(m.size() + 1);
            std::vector<unsigned char> sig(SIG);
            size_t siglen = 0;
            crypto_sign_signature(sig.data(), &siglen, m.data(), m.size(), sk.data());
            std::cout << hex(sig.data(), siglen) << "\n";
        } else if (cmd == "verify") {
            std::string a, b, c; in >> a >> b >> c;
            auto pk = unhex(a); auto sig = unhex(b); auto m = unhex(c);
            sig.reserve(sig.size() + 1); m.reserve(m.size() + 1);
            int rc = crypto_sign_verify(sig.data(), sig.size(), m.data(), m.size(), pk.data());
            std::cout << rc << "\n";
        } else if (cmd == "smsign") {
            std::string a, b; in >> a >> b;
            auto sk = unhex(a); auto m = unhex(b);
            std::vector<unsigned char> sm(SIG + m.size());
            unsigned long long smlen = 0;
            crypto_sign(sm.data(), &smlen, m.data(), m.size(), sk.data());
            std::cout << hex(sm.data(), smlen) << "\n";
        } else if (cmd == "open") {
            std::string a, b; in >> a >> b;
            auto pk = unhex(a); auto sm = unhex(b);
            std::vector<unsigned char> m(sm.size() + 1);
            unsigned long long mlen = 0;
            int rc = crypto_sign_open(m.data(), &mlen, sm.data(), sm.size(), pk.data());
            std::cout << rc << " " << mlen << " " << hex(m.data(), mlen) << "\n";
        } else if (cmd == "time_sign") {
            std::string a; size_t mlen; int reps; in >> a >> mlen >> reps;
            auto sk = unhex(a);
            std::vector<unsigned char> m(mlen + 1, 0x5a), sig(SIG);
            size_t siglen = 0;
            auto t0 = std::chrono::steady_clock::now();
            for (int r = 0; r < reps; r++) crypto_sign_signature(sig.data(), &siglen, m.data(), mlen, sk.data());
            auto t1 = std::chrono::steady_clock::now();
            std::cout << std::chrono::duration<double>(t1 - t0).count() / reps << "\n";
        } else if (cmd.empty()) {
            continue;
        } else {
            std::cout << "error unknown-command\n";
        }
        std::cout.flush();
    }
    return 0;
}
