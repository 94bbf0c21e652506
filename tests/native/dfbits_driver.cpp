// CPU driver for the integer float/double conversions of csrc/dfbits.cuh:
//   split:  reads doubles from stdin, writes (ok, hi bits, lo bits) per value
//   rint:   reads (double, int64 sh) pairs, writes (ok, int64 value)
//   absmax: reads doubles, writes the bits of the largest |x| (NaNs skipped)
#include <cstdio>
#include <cstring>
#include <vector>
#include "../../modal-cmb_gb300/csrc/dfbits.cuh"

int main(int argc, char **argv)
{
    if (argc < 2) return 2;
    if (!strcmp(argv[1], "split")) {
        double x;
        while (fread(&x, 8, 1, stdin) == 1) {
            uint32_t h = 0, l = 0, ok = dfb::split(x, &h, &l) ? 1u : 0u;
            uint32_t o[3] = {ok, h, l};
            fwrite(o, 4, 3, stdout);
        }
        return 0;
    }
    if (!strcmp(argv[1], "rint")) {
        struct { double x; int64_t sh; } in;
        while (fread(&in, 16, 1, stdin) == 1) {
            long long F = 0;
            int64_t o[2] = {dfb::scaled_rint(in.x, (int)in.sh, &F) ? 1 : 0, (int64_t)F};
            fwrite(o, 8, 2, stdout);
        }
        return 0;
    }
    if (!strcmp(argv[1], "absmax")) {
        double x;
        uint64_t m = 0;
        while (fread(&x, 8, 1, stdin) == 1) m = dfb::absmax_bits(m, x);
        fwrite(&m, 8, 1, stdout);
        return 0;
    }
    return 2;
}
