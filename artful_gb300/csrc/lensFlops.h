/* artful_cuda — the algorithmic work of a trace, for the roofline.
 *
 * Counting rule: each float + - * / sqrt min max is one operation (a fused multiply-add two; a
 * reciprocal square root a square root and a division); comparisons, floor, abs, sign flips,
 * conversions, integer work and loads are not counted.  The constants are an exact count of the
 * formulas in lensCore.cuh: tests/flops_count.cpp evaluates those formulas on the host with an
 * operation-counting number type and tests/test_flops.py checks every constant here against it.
 *
 *   per ray      the set-up of the constants of motion and the first state (rayStart, the first drag,
 *                the disc's radial scale); the 15 products of the ray's constants that each Nystrom
 *                sub-step's formulas recompute (a^2, h^2, h/2, h^2/8, h^2/2, h^2/6, h/6 in both, 2a^2 in
 *                the polar one), counted once a ray since they do not change along it; and the 3 sums
 *                that add the ray's light to its pixel (the pixel's 3 products by 1 / rays not counted)
 *   per step     one Nystrom step with its frame-drag terms (spin != 0), without those 15, and the
 *                plane test n_z n_z'
 *   per crossing an accepted crossing's position, three slices of the disc (all inside), the ring's
 *                heat and glow, the Doppler shift (doppler != 0) and the colour
 *   per escape   the escape point and the direction in the sky's frame; with stars > 0, the stars and
 *                sky dust toward it where neither star layer draws a star there (a drawn star adds up to
 *                63 more: counted as none, so the count is a lower bound there) */
#pragma once

#define ARTF_FLOPS_RAY 100
#define ARTF_FLOPS_RAY_SPINLESS 88     /* spin 0: no initial drag */
#define ARTF_FLOPS_STEP 149
#define ARTF_FLOPS_STEP_SPINLESS 122   /* spin 0: no drag, no psi */
#define ARTF_FLOPS_CROSSING 375
#define ARTF_FLOPS_CROSSING_DOPPLER 26 /* of those, the Doppler shift's */
#define ARTF_FLOPS_ESCAPE 59
#define ARTF_FLOPS_SKY 58

/* The mixed trace's wide work, the operations it carries at about FP64's precision, by the same rule:
 * double-float pairs on the FP32 pipe, but for the horizon's band, which runs in FP64.
 *   per set-up   a ray's constants of motion (what it takes from its view formed once a view; its first
 *                state and step are FP32 work), and its step's terms (formed once a ray)
 *   per horizon  one whole radial sub-step (u, du/ds and psi) with those terms given, in the horizon's
 *                band; spin 0: no drag, no psi
 *   per turn     the radial motion alone (u, du/ds), at a turning point of u
 *   per polar    the polar axis component alone (n_z, dn_z/ds), at a turning point of n_z */
#define ARTF_FLOPS_WIDE_START 51
#define ARTF_FLOPS_WIDE_RADIAL 61
#define ARTF_FLOPS_WIDE_RADIAL_SPINLESS 34
#define ARTF_FLOPS_WIDE_TURN 34
#define ARTF_FLOPS_WIDE_AXIS 37

static inline double artfFlops64(unsigned long long setups, unsigned long long horizon, unsigned long long turns,
                                 unsigned long long polar, int spinning) {
    return ARTF_FLOPS_WIDE_START * (double)setups +
           (spinning ? ARTF_FLOPS_WIDE_RADIAL : ARTF_FLOPS_WIDE_RADIAL_SPINLESS) * (double)horizon +
           ARTF_FLOPS_WIDE_TURN * (double)turns + ARTF_FLOPS_WIDE_AXIS * (double)polar;
}

static inline double artfFlops(unsigned long long rays, unsigned long long steps, unsigned long long crossings,
                               unsigned long long escapes, int spinning, int doppler, int stars) {
    const double perRay = spinning ? ARTF_FLOPS_RAY : ARTF_FLOPS_RAY_SPINLESS;
    const double perStep = spinning ? ARTF_FLOPS_STEP : ARTF_FLOPS_STEP_SPINLESS;
    const double perCrossing = ARTF_FLOPS_CROSSING - (doppler ? 0 : ARTF_FLOPS_CROSSING_DOPPLER);
    const double perEscape = ARTF_FLOPS_ESCAPE + (stars ? ARTF_FLOPS_SKY : 0);
    return perRay * (double)rays + perStep * (double)steps + perCrossing * (double)crossings +
           perEscape * (double)escapes;
}
