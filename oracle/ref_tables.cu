// ref_tables.cu — dumps the reference's own per-spin tables.
//
// TEST INFRASTRUCTURE ONLY: this driver #includes the reference project's
// MBL_test/include/fermi_operator.h unmodified (from the read-only reference
// checkout, path given to the compiler with -I by oracle/Makefile) and runs
// its H_TBq builder, so the fixtures in tests/golden/ carry the reference's
// exact basis (H_TBq::state/address, fermi_operator.h:44-53) and ELL tables
// (H_TBq::Ax/Aj built by Make_H/Make_J/Make_N, fermi_operator.h:100-149).
//
// Input (stdin, whitespace separated):
//   N Q
//   then any number of operations, one per line:
//     H i j t     -> Hq.Make_H(i, j, t)
//     J i j t     -> Hq.Make_J(i, j, t)
//     N i v       -> Hq.Make_N(i, v)
//   terminated by "E".
// Output (stdout, little-endian binary):
//   int32 count, int32 nslots,
//   int32 state[count], int32 address[2^N],
//   float64 Ax[nslots*count], int32 Aj[nslots*count]
#include <cstdio>
#include <cstdint>
#include <iostream>
#include <string>
#include "fermi_operator.h"

int main() {
    int N, Q;
    if (!(std::cin >> N >> Q)) return 2;
    H_TBq hq(N, Q);
    std::string op;
    while (std::cin >> op) {
        if (op == "E") break;
        if (op == "H" || op == "J") {
            int i, j; double t;
            std::cin >> i >> j >> t;
            if (op == "H") hq.Make_H(i, j, t); else hq.Make_J(i, j, t);
        } else if (op == "N") {
            int i; double v;
            std::cin >> i >> v;
            hq.Make_N(i, v);
        } else {
            return 3;
        }
    }
    int32_t count = hq.count, nslots = z * Q + 1;
    fwrite(&count, 4, 1, stdout);
    fwrite(&nslots, 4, 1, stdout);
    for (int a = 0; a < count; ++a) { int32_t s = hq.state[a]; fwrite(&s, 4, 1, stdout); }
    for (int n = 0; n < (1 << N); ++n) {
        int32_t a = (__builtin_popcount(n) == Q) ? hq.address[n] : -1;
        fwrite(&a, 4, 1, stdout);
    }
    for (size_t k = 0; k < (size_t)nslots * count; ++k) { double v = hq.Ax[k]; fwrite(&v, 8, 1, stdout); }
    for (size_t k = 0; k < (size_t)nslots * count; ++k) { int32_t j = hq.Aj[k]; fwrite(&j, 4, 1, stdout); }
    return 0;
}
