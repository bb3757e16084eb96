// Generates golden values of the reference's host-callable helpers
// (asph_h100.cu:136-171: theta_ref, exner_ref, pres_ref, rho_ref, qv_ref,
// esat, qsat, dqsdT) by compiling the reference file itself for the host
// and calling them.  Built and run by tests/golden/make_golden.py where the
// reference checkout exists; the values are committed as a fixture.
#define main asph_reference_main
#include REFSRC
#undef main
#include <cstdio>

int main(int argc, char** argv) {
    if (argc != 2) return 1;
    FILE* f = fopen(argv[1], "wb");
    if (!f) return 1;
    for (int i = 0; i <= 200; ++i) {
        float z = 75.0f * (float)i;                 // 0 .. 15 km
        float T = 200.0f + 0.5f * (float)i;         // 200 .. 300 K
        float p = 30000.0f + 350.0f * (float)i;     // 300 .. 1000 hPa
        float v[9] = {z, theta_ref(z), exner_ref(z), pres_ref(z), rho_ref(z), qv_ref(z), esat(T), qsat(T, p),
                      dqsdT(T, esat(T), p)};
        fwrite(v, sizeof(float), 9, f);
        float tp[2] = {T, p};
        fwrite(tp, sizeof(float), 2, f);
    }
    fclose(f);
    return 0;
}
