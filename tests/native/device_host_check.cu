// Host-side check of imc_device.cuh (the __host__ __device__ paths): reads
// commands on stdin, prints results on stdout.  Built and driven by
// tests/test_device_header.py; needs no GPU.
//   P c0 c1 c2 c3 k0 k1          -> philox4x32_10 words
//   S seed step pid stage n      -> n words of a Stream
//   F b v1 v2 ... (until '.')    -> exact fixed-point total of the values, as
//                                   signed limb sums "a0 a1 a2" and the double
//   R prec n v1..vn K s1..sK     -> sorter<prec> product (hex) and scale index
//   W b v1 v2 ... (until '.')    -> per FP32 value: "1 l0 l1 l2" from f32_words
//                                   (words as the signed limbs of fix_split),
//                                   "0" where f32_words declines, and
//                                   fix_split's "ok l0 l1 l2" after it
//   A                            -> the m < 2^24 where two_pi_u24(m) differs
//                                   from (float)(2 pi * (double)(m 2^-24)),
//                                   then "done <count>"
//   B                            -> the m < 2^24 where a 2D surface-birth angle
//                                   from pi_n24 differs from the Float64 form
//                                   (faces 1 and 2), then "done <count>"
//   C                            -> the binary32 x >= 0 (and +inf) where
//                                   cutoff_energy(x) differs from
//                                   (float)(0.01 * (double)x), "done <count>"
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <iostream>
#include <sstream>
#include <vector>
#include "../../mixedprecisionimc.jl_gb300/csrc/imc_device.cuh"

using namespace imc;

int main() {
    std::string line;
    while (std::getline(std::cin, line)) {
        std::istringstream in(line);
        std::string cmd;
        in >> cmd;
        if (cmd == "P") {
            uint32_t c[4], k[2], o[4];
            in >> c[0] >> c[1] >> c[2] >> c[3] >> k[0] >> k[1];
            philox4x32_10(c[0], c[1], c[2], c[3], k[0], k[1], o);
            printf("%u %u %u %u\n", o[0], o[1], o[2], o[3]);
        } else if (cmd == "S") {
            unsigned long long seed; uint32_t step, pid, stage; int n;
            in >> seed >> step >> pid >> stage >> n;
            Stream s; s.init(seed, step, pid, stage);
            for (int i = 0; i < n; ++i) printf("%u%c", s.next(), i + 1 < n ? ' ' : '\n');
        } else if (cmd == "F") {
            int b; in >> b;
            long long acc[3] = {0, 0, 0};
            std::string tok;
            bool ok = true;
            while (in >> tok && tok != ".") {
                double v = strtod(tok.c_str(), nullptr);
                Limbs L;
                bool r = (tok.back() == 'f') ? fix_split((float)v, b, L) : fix_split(v, b, L);
                if (!r) { ok = false; continue; }
                acc[0] += L.l0; acc[1] += L.l1; acc[2] += L.l2;
            }
            printf("%d %lld %lld %lld %.17g\n", ok ? 1 : 0, acc[0], acc[1], acc[2], fix_value(acc, b));
        } else if (cmd == "W") {
            int b; in >> b;
            std::string tok;
            while (in >> tok && tok != ".") {
                const float v = strtof(tok.c_str(), nullptr);
                int j; uint32_t lo, hi;
                long long w[3] = {0, 0, 0};  // bits 0-31, 32-63, 64-95
                const bool f = f32_words(v, b, j, lo, hi);
                if (f) { w[j] = lo; if (j < 2) w[j + 1] = hi; else if (hi) w[0] = -1; }
                Limbs L;
                const bool r = fix_split(v, b, L);
                printf("%d %lld %lld %lld %d %lld %lld %lld\n", f ? 1 : 0, w[2], w[1], w[0], r ? 1 : 0,
                       r ? L.l0 : 0, r ? L.l1 : 0, r ? L.l2 : 0);
            }
        } else if (cmd == "A") {
            const double two_pi = 2.0 * 3.141592653589793;
            long bad = 0;
            for (uint32_t m = 0; m < (1u << 24); ++m) {
                const float ref = (float)(two_pi * (double)((float)m * 0x1p-24f));
                const float got = two_pi_u24(m);
                if (std::memcmp(&ref, &got, 4) != 0) {
                    if (bad < 8) printf("%u ", m);
                    ++bad;
                }
            }
            printf("done %ld\n", bad);
        } else if (cmd == "B") {
            const double pd = 3.141592653589793;
            long bad = 0;
            for (uint32_t m = 0; m < (1u << 24); ++m) {
                const float u = (float)m * 0x1p-24f;
                const float r1 = (float)(-pd * (double)u), g1 = -pi_n24((int)m);
                const float r2 = (float)(pd * (0.5 - (double)u)), g2 = pi_n24((1 << 23) - (int)m);
                if (std::memcmp(&r1, &g1, 4) || std::memcmp(&r2, &g2, 4)) {
                    if (bad < 8) printf("%u ", m);
                    ++bad;
                }
            }
            printf("done %ld\n", bad);
        } else if (cmd == "C") {
            long bad = 0;
            for (uint32_t b = 0; b <= 0x7F800000u; ++b) {
                float x;
                std::memcpy(&x, &b, 4);
                const float ref = (float)(0.01 * (double)x);
                const float got = cutoff_energy(x);
                if (std::memcmp(&ref, &got, 4) != 0) {
                    if (bad < 8) printf("%a ", x);
                    ++bad;
                }
            }
            printf("done %ld\n", bad);
        } else if (cmd == "R") {
            int prec, n, K;
            in >> prec >> n;
            // values as strtod tokens, so nan, inf and -0.0 pass through
            std::string t;
            std::vector<double> v(n);
            for (auto &x : v) { in >> t; x = strtod(t.c_str(), nullptr); }
            in >> K;
            std::vector<double> s(K);
            for (auto &x : s) { in >> t; x = strtod(t.c_str(), nullptr); }
            int j;
            double p = prec == 0 ? sorter<0>(v.data(), n, s.data(), K, &j)
                     : prec == 1 ? sorter<1>(v.data(), n, s.data(), K, &j)
                                 : sorter<2>(v.data(), n, s.data(), K, &j);
            printf("%a %d\n", p, j);
        }
        fflush(stdout);
    }
    return 0;
}
