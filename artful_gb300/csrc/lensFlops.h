/* artful_cuda — the algorithmic work of a trace, for the roofline.
 *
 * Counting rule: each float + - * / sqrt min max is one operation (a fused multiply-add two);
 * comparisons, floor, abs, conversions, integer work and loads are not counted; loop-invariant
 * products the compiler hoists are counted once per ray.  The constants are an exact count of the
 * formulas in lensCore.cuh (tests/test_flops.py evaluates those formulas on the host with an
 * operation-counting number type and checks every constant here).
 *
 *   per ray      setup of the constants of motion and the first state (rayStart, the first drag, the
 *                disc's radial scale), and the pixel's sum
 *   per step     one Nystrom step with its frame-drag terms (spin != 0), and the plane test
 *   per crossing the crossing's position, three slices of the disc, the ring's heat and glow, the
 *                Doppler shift (doppler != 0) and the colour
 *   per escape   the escape direction, and the stars and sky dust (stars > 0) */
#pragma once

#define ARTF_FLOPS_RAY 85
#define ARTF_FLOPS_RAY_SPINLESS 74     /* spin 0: no initial drag */
#define ARTF_FLOPS_STEP 149
#define ARTF_FLOPS_STEP_SPINLESS 122   /* spin 0: no drag, no psi */
#define ARTF_FLOPS_CROSSING 395
#define ARTF_FLOPS_CROSSING_DOPPLER 26 /* of those, the Doppler shift's */
#define ARTF_FLOPS_ESCAPE 63
#define ARTF_FLOPS_SKY 61

static inline double artfFlops(unsigned long long rays, unsigned long long steps, unsigned long long crossings,
                               unsigned long long escapes, int spinning, int doppler, int stars) {
    const double perRay = spinning ? ARTF_FLOPS_RAY : ARTF_FLOPS_RAY_SPINLESS;
    const double perStep = spinning ? ARTF_FLOPS_STEP : ARTF_FLOPS_STEP_SPINLESS;
    const double perCrossing = ARTF_FLOPS_CROSSING - (doppler ? 0 : ARTF_FLOPS_CROSSING_DOPPLER);
    const double perEscape = ARTF_FLOPS_ESCAPE + (stars ? ARTF_FLOPS_SKY : 0);
    return perRay * (double)rays + perStep * (double)steps + perCrossing * (double)crossings +
           perEscape * (double)escapes;
}
