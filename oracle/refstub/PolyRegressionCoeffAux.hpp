// Placeholder for the reference's missing coefficient table. Only the
// 2nd-order polynomial regression predictor reads it, which no build of the
// interpolation path reaches; the arrays are one element so the header compiles.
#pragma once
static float COEFF_1D[1] = {0.f};
static float COEFF_2D[1] = {0.f};
static float COEFF_3D[1] = {0.f};
