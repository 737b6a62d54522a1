// spx_sets.h -- the runtime parameter-set table (host side).
//
// The reference fixes one parameter set per build (params.h:4-79, Makefile
// -D flags at Makefile:109-155); here every set is a row of this table and
// the device code is instantiated per (hash, n, robust).
#pragma once
#include <stdint.h>
#include <string.h>

namespace cuspx {

struct SetDesc {
    const char *name;   // e.g. "sha256-128f-simple"
    int hash;           // 0 sha256, 1 shake256
    int robust;         // 0 simple, 1 robust
    int n, h, d, a, k;
};

// 6 sizes x 2 hash families x simple/robust.  Ids are the row index.
static const SetDesc kSets[] = {
    {"sha256-128s-simple", 0, 0, 16, 63, 7, 12, 14},   {"sha256-128s-robust", 0, 1, 16, 63, 7, 12, 14},
    {"sha256-128f-simple", 0, 0, 16, 66, 22, 6, 33},   {"sha256-128f-robust", 0, 1, 16, 66, 22, 6, 33},
    {"sha256-192s-simple", 0, 0, 24, 63, 7, 14, 17},   {"sha256-192s-robust", 0, 1, 24, 63, 7, 14, 17},
    {"sha256-192f-simple", 0, 0, 24, 66, 22, 8, 33},   {"sha256-192f-robust", 0, 1, 24, 66, 22, 8, 33},
    {"sha256-256s-simple", 0, 0, 32, 64, 8, 14, 22},   {"sha256-256s-robust", 0, 1, 32, 64, 8, 14, 22},
    {"sha256-256f-simple", 0, 0, 32, 68, 17, 9, 35},   {"sha256-256f-robust", 0, 1, 32, 68, 17, 9, 35},
    {"shake256-128s-simple", 1, 0, 16, 63, 7, 12, 14}, {"shake256-128s-robust", 1, 1, 16, 63, 7, 12, 14},
    {"shake256-128f-simple", 1, 0, 16, 66, 22, 6, 33}, {"shake256-128f-robust", 1, 1, 16, 66, 22, 6, 33},
    {"shake256-192s-simple", 1, 0, 24, 63, 7, 14, 17}, {"shake256-192s-robust", 1, 1, 24, 63, 7, 14, 17},
    {"shake256-192f-simple", 1, 0, 24, 66, 22, 8, 33}, {"shake256-192f-robust", 1, 1, 24, 66, 22, 8, 33},
    {"shake256-256s-simple", 1, 0, 32, 64, 8, 14, 22}, {"shake256-256s-robust", 1, 1, 32, 64, 8, 14, 22},
    {"shake256-256f-simple", 1, 0, 32, 68, 17, 9, 35}, {"shake256-256f-robust", 1, 1, 32, 68, 17, 9, 35},
};
static const int kNumSets = (int)(sizeof(kSets) / sizeof(kSets[0]));

inline int set_by_name(const char *name) {
    for (int i = 0; i < kNumSets; i++)
        if (!strcmp(kSets[i].name, name)) return i;
    // a bare "<hash>-<size>" names the simple set, as the reference builds do
    for (int i = 0; i < kNumSets; i++)
        if (!kSets[i].robust && !strncmp(kSets[i].name, name, strlen(name)) && strlen(name) + 7 == strlen(kSets[i].name))
            return i;
    return -1;
}

}  // namespace cuspx
