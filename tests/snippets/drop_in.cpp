/* A small program over the C++ layer: parses a ddplan, writes Boxcar::dump2txt on host-filled
 * planes, and with an argument searches four synthetic blocks end to end on the GPU. */
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include "transientx_gb300.hpp"
int main(int argc, char **argv) {
    const int C = 64; const long N = 2048; const double tsamp = 256e-6;
    std::vector<double> f(C);
    for (int j = 0; j < C; j++) f[j] = 1500.0 - (j + 0.5) * 300.0 / C;
    auto rows = txgpu::parse_ddplan("# td fd dms ddm ndm snrloss maxw\n1 1 0 1 100 0.1 0.02\n");
    rows[0].nsub = 8;
    if (argc < 2) {
        std::printf("parsed %zu rows\n", rows.size());
        txgpu::Boxcar bx;                 /* Boxcar::dump2txt on host-filled planes */
        bx.ndm = 3;
        bx.nsamples = 4;
        for (int k = 0; k < 12; k++) bx.mxS.push_back(k * 1.25f - 3.5f);
        bx.dump2txt("boxcar.txt");
        txgpu::Boxcar none;
        none.ndm = 2;
        none.nsamples = 2;
        try { none.dump2txt("never.txt"); std::printf("no throw\n"); }
        catch (const txgpu::Error &e) { std::printf("throws %d\n", e.status); }
        return 0;
    }
    txgpu::Search s(rows, C, tsamp, f, N);
    std::vector<uint8_t> raw(N * C);
    unsigned long long z = 12345;
    int found = 0;
    for (int b = 0; b < 4; b++) {
        for (long t = 0; t < N; t++)
            for (int j = 0; j < C; j++) {
                double g = 0; for (int k = 0; k < 12; k++) { z = z * 6364136223846793005ULL + 1442695040888963407ULL; g += (z >> 11) * (1.0 / 9007199254740992.0); }
                double v = 128 + 12 * (g - 6);
                long tt = b * N + t;
                double d = 4.148741601e3 * 50.0 * (1.0 / (f[j] * f[j]) - 1.0 / (f[0] * f[0])) / tsamp;
                if (tt >= 5000 + std::lround(d) && tt < 5008 + std::lround(d)) v += 30;
                raw[t * C + j] = (uint8_t)std::fmin(255, std::fmax(0, std::floor(v + 0.5)));
            }
        s.run(raw.data());
        s.sync();
        if (s.info(0).gated) found += (int)s.cluster(0).size();
    }
    std::printf("clusters %d\n", found);
    return found > 0 ? 0 : 1;
}
