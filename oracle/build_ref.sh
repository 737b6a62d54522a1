#!/usr/bin/env bash
# Build the reference's own CPU SPHINCS+ path, per parameter set, straight
# from the reference sources where they lie, into oracle/_ref/<set>/.
#
# Test infrastructure only (the product never links it).  The reference is
# CUDA C++ (.cu files mixing host and device code), so nvcc compiles it; only
# host entry points are ever called and no GPU is needed.  The one external
# dependency is AES-256-ECB from the system libcrypto.so.3 (rng.cu:116-136);
# oracle/shim/openssl declares the five prototypes rng.cu uses because the
# OpenSSL development headers are absent.  Compile flags follow the
# reference's own per-variant flags (Makefile:109-155: -DVARIANT -D<hash>
# -D<set> -DSIMPLE, -O3, relocatable device code).
#
# usage: oracle/build_ref.sh [--release] [--if-present] [set ...]
#        set = sha256-128f, shake256-256f, ...
#        REF=/path/to/reference (default /root/reference)
#
# --release builds the reference's release behaviour into
# oracle/_ref/<set>-release/: as shipped, all_option.h defines DEBUG_MODE,
# which replaces crypto_sign_keypair's DRBG seed by 0..3n-1 (sign.cu:346-349)
# and crypto_sign_signature's DRBG optrand by 0xAD bytes (sign.cu:1951-1954).
# The sources include "all_option.h" from their own directory, so an include
# path cannot shadow it: the sources are copied into oracle/_ref/src-release/
# (git-ignored build input, never committed) with that one #define line
# deleted, and compiled from there.  Only the ref_golden driver is built.
#
# --if-present exits 0 without building when the reference tree is absent
# (the case on a machine that only runs the prebuilt tests).
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${REF:-/root/reference}"
OUT="$HERE/_ref"
RELEASE=0
IF_PRESENT=0
while [ $# -gt 0 ]; do
    case "$1" in
        --release) RELEASE=1; shift;;
        --if-present) IF_PRESENT=1; shift;;
        *) break;;
    esac
done
ARCH="${REF_ARCH:-sm_100}"
SOURCES="common.cu address.cu rng.cu wots.cu utils.cu fors.cu sign.cu fips202.cu gpu_fips202.cu hash_shake256.cu thash_shake256.cu sha256.cu gpu_sha256.cu hash_sha256.cu thash_sha256.cu"
LIBCRYPTO="${LIBCRYPTO:-$(ls /usr/lib/*-linux-gnu/libcrypto.so.3 2>/dev/null | head -1)}"

if [ ! -d "$REF" ]; then
    [ "$IF_PRESENT" = 1 ] && exit 0
    echo "reference sources not found at $REF" >&2; exit 2
fi
if [ -z "$LIBCRYPTO" ]; then echo "libcrypto.so.3 not found" >&2; exit 2; fi
SETS="$*"
[ -z "$SETS" ] && SETS="sha256-128f"

build_one() {
    local set="$1" hash size hdef sdef dir
    hash="${set%%-*}"; size="${set##*-}"
    case "$hash" in sha256) hdef=SHA256;; shake256) hdef=SHAKE256;; *) echo "bad set $set" >&2; return 2;; esac
    sdef="SPX_$(echo "$size" | tr a-z A-Z)"
    dir="$OUT/$set"
    if [ -x "$dir/ref_golden" ] && [ -x "$dir/PQCgenKAT_sign" ] && [ "$dir/ref_golden" -nt "$HERE/ref_golden.cu" ]; then return 0; fi
    mkdir -p "$dir"
    local flags="-ccbin g++ --expt-relaxed-constexpr -O3 -m64 -dc -arch=$ARCH -w -I$HERE/shim -I$REF -DVARIANT -D$hdef -D$sdef -DSIMPLE"
    local objs=""
    for s in $SOURCES; do
        nvcc $flags -o "$dir/${s%.cu}.o" "$REF/$s" &
        objs="$objs $dir/${s%.cu}.o"
    done
    nvcc $flags -o "$dir/ref_golden.o" "$HERE/ref_golden.cu" &
    nvcc $flags -o "$dir/PQCgenKAT_sign.o" "$REF/PQCgenKAT_sign.cu" &
    wait
    nvcc -arch=$ARCH -o "$dir/ref_golden" $objs "$dir/ref_golden.o" -Xlinker "$LIBCRYPTO" -lstdc++ -lm
    # the reference's own NIST KAT generator (PQCgenKAT_sign.cu), same objects
    nvcc -arch=$ARCH -o "$dir/PQCgenKAT_sign" $objs "$dir/PQCgenKAT_sign.o" -Xlinker "$LIBCRYPTO" -lstdc++ -lm
}

# release behaviour: a copy of the sources without the DEBUG_MODE define
build_release() {
    local set="$1" hash size hdef sdef dir src="$OUT/src-release"
    hash="${set%%-*}"; size="${set##*-}"
    case "$hash" in sha256) hdef=SHA256;; shake256) hdef=SHAKE256;; *) echo "bad set $set" >&2; return 2;; esac
    sdef="SPX_$(echo "$size" | tr a-z A-Z)"
    dir="$OUT/$set-release"
    if [ -x "$dir/ref_golden" ] && [ "$dir/ref_golden" -nt "$HERE/ref_golden.cu" ] && [ "$dir/ref_golden" -nt "$HERE/build_ref.sh" ]; then return 0; fi
    mkdir -p "$src" "$dir"
    cp "$REF"/*.cu "$REF"/*.h "$src/"
    sed -i '/^[[:space:]]*#define[[:space:]]\+DEBUG_MODE[[:space:]]*$/d' "$src/all_option.h"
    if grep -q "define[[:space:]]*DEBUG_MODE" "$src/all_option.h"; then echo "DEBUG_MODE still defined" >&2; return 2; fi
    local flags="-ccbin g++ --expt-relaxed-constexpr -O3 -m64 -dc -arch=$ARCH -w -I$HERE/shim -I$src -DVARIANT -D$hdef -D$sdef -DSIMPLE"
    local objs=""
    for s in $SOURCES; do
        nvcc $flags -o "$dir/${s%.cu}.o" "$src/$s" &
        objs="$objs $dir/${s%.cu}.o"
    done
    nvcc $flags -o "$dir/ref_golden.o" "$HERE/ref_golden.cu" &
    wait
    nvcc -arch=$ARCH -o "$dir/ref_golden" $objs "$dir/ref_golden.o" -Xlinker "$LIBCRYPTO" -lstdc++ -lm
}

for s in $SETS; do
    if [ "$RELEASE" = 1 ]; then build_release "$s"; else build_one "$s"; fi
done
