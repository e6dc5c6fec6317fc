/* Exercises the library's host C11 code (holeHost.c, synthScene.c) over ordinary and edge inputs, built by
 * tests/test_host_sanitized.py with AddressSanitizer and UndefinedBehaviorSanitizer: any out-of-bounds
 * access, leak, signed overflow, misaligned or null access stops it with a report and a non-zero exit.
 * Prints a checksum of what it computed, so nothing is optimised away. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "artful_cuda.h"

static double sum;

static void add(double x) {
    if (isfinite(x)) sum += x;
}

static void take(const void* p, size_t bytes) {
    const unsigned char* b = (const unsigned char*)p;
    for (size_t i = 0; i < bytes; ++i) sum += b[i];
}

static ArtfCudaCamera camera(float inclinationDeg, float r) {
    const float i = inclinationDeg * 3.14159265f / 180.f;
    ArtfCudaCamera c;
    memset(&c, 0, sizeof c);
    c.position.x = 0.f, c.position.y = r * cosf(i), c.position.z = r * sinf(i);
    c.up.y = 1.f;
    c.fovY = .6f;
    c.near_ = .1f;
    return c;
}

int main(void) {
    const float spins[] = {-1.5f, -0.998f, 0.f, 0.3f, 0.9f, 0.998f, 1.f, 2.f, NAN};
    const float incl[] = {0.f, 5.f, 60.f, 85.f, 90.f, 179.f};
    const int sizes[][2] = {{1, 1}, {3, 2}, {101, 67}, {320, 180}};
    ArtfCudaBlackHoleDesc d = artfCudaBlackHoleDefaults();
    for (size_t s = 0; s < sizeof spins / sizeof *spins; ++s) {
        add(artfCudaIsco(spins[s]));
        add(artfCudaOrbitSpeed(spins[s], 6.f));
        ArtfCudaBlackHoleDesc in = d, out;
        in.axis.y = 1.f;
        in.spin = spins[s];
        in.discInner = s % 2 ? 0.f : -3.f;
        in.discOuter = s % 3 ? 12.f : 1e9f;
        in.samples = (int)s - 2;
        in.discHeight = s % 2 ? 1e-6f : 5.f;
        artfCudaHoleClamp(&in, &out);
        take(&out, sizeof out);
        for (size_t k = 0; k < sizeof incl / sizeof *incl; ++k)
            for (size_t z = 0; z < sizeof sizes / sizeof *sizes; ++z) {
                const ArtfCudaCamera c = camera(incl[k], 30.f);
                ArtfCudaHoleFrame f;
                ArtfCudaHoleFrame64 f64;
                sum += artfCudaHoleFrame(&c, &out, 1.5, sizes[z][0], sizes[z][1], &f);
                sum += artfCudaHoleFrame64(&c, &out, 1.5, sizes[z][0], sizes[z][1], &f64);
                take(&f, sizeof f);
                take(&f64, sizeof f64);
            }
    }
    /* refused arguments */
    ArtfCudaHoleFrame f;
    sum += artfCudaHoleFrame(NULL, &d, 0.0, 4, 4, &f) + artfCudaHoleFrame(NULL, NULL, 0.0, 0, -1, NULL);
    double clock = 0.0;
    const double times[] = {0.0, 0.1, 0.21, 30.0, 29.0, 5.0, -4.0, 1e9};
    for (size_t t = 0; t < sizeof times / sizeof *times; ++t) {
        add(artfCudaFluidClock(&clock, times[t]));
        add(clock);
    }
    /* the parameter scenes and their frames, Jacobians and maps */
    float* map = (float*)malloc(sizeof(float) * ARTF_CUDA_MAP_FLOATS);
    if (!map) return 2;
    const ArtfCudaHoleParams params[] = {
        {0.7, 1.047, 1.0, 3.0, 30.0, 0.6, 12.0, 1e-3, 0.0, 1.0, 1.0, 1.0, 0.0, 4},
        {0.0, 0.1, 0.5, 2.0, 4.0, 0.6, 20.0, 1e-3, 0.0, 1.0, 0.0, 0.0, 3.0, 1},
        {0.997, 3.0, 1.5, 3.5, 80.0, 0.6, 12.0, 1e-3, 0.0, 1.0, 1.0, 1.0, 0.0, 7},
        {1.5, -1.0, -2.0, 3.0, 1.0, 0.6, 12.0, 1e-3, 0.0, 1.0, 1.0, 1.0, 0.0, 9}, /* out of range: refused */
    };
    for (size_t p = 0; p < sizeof params / sizeof *params; ++p) {
        ArtfCudaCamera c;
        ArtfCudaBlackHoleDesc desc;
        ArtfCudaHoleFrame f32;
        ArtfCudaHoleFrame64 f64;
        double jacobian[ARTF_CUDA_GRAD_FIELDS * 5];
        sum += artfCudaHoleParamsScene(&params[p], &c, &desc);
        sum += artfCudaHoleParamsFrames(&params[p], 37, 21, &f32, &f64, jacobian);
        if (artfCudaHoleParamsMap(&params[p], map) == 0) take(map, sizeof(float) * 4096);
        for (int k = 0; k < ARTF_CUDA_GRAD_FIELDS * 5; ++k) sum += isfinite(jacobian[k]) ? 0.0 : 1.0;
    }
    /* synthetic maps over discs and seeds */
    const ArtfCudaSynthDesc synth[] = {{0, 1.237f, 12.f, .998f, 3.f, 2000}, {3, 6.f, 12.f, 0.f, 2.7f, 0},
                                       {~0ull, 2.f, 50.f, .5f, 0.f, 5}};
    for (size_t s = 0; s < sizeof synth / sizeof *synth; ++s) {
        sum += artfCudaSynthMap(&synth[s], map);
        artfCudaSynthRings(&synth[s], map);
        take(map + ARTF_CUDA_MAP_FLOATS - 1024, sizeof(float) * 1024);
    }
    free(map);
    printf("checksum %.6g\n", sum);
    return 0;
}
