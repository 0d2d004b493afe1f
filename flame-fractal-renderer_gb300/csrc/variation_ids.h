// Variation identifiers.  The id order is the reference's factory order:
// the 20 N-dimensional names of Variation::parseVariationNd
// (src/variations/variations.hpp:2567-2612), then the 78 two-dimensional
// names of Variation::parseVariation2d (variations.hpp:2387-2548).  The
// three-dimensional factory is empty (variations.hpp:2559-2564).
#pragma once

#include "std_types.h"

namespace ffr {

enum VariationId : int32_t
{
    // N-D
    V_LINEAR = 0, V_SINUSOIDAL, V_SPHERICAL, V_BENT, V_RECTANGLES, V_FISHEYE,
    V_BUBBLE, V_NOISE, V_BLUR, V_GAUSSIAN_BLUR, V_SQUARE_NOISE, V_SEPARATION,
    V_SPLITS, V_PRE_BLUR, V_MODULUS, V_CELLN, V_SPHERICAL_P, V_UNIT_SPHERE,
    V_UNIT_SPHERE_P, V_UNIT_CUBE,
    // 2-D (VariationFrom2D, variations.hpp:63-107)
    V_SWIRL, V_HORSESHOE, V_POLAR, V_POLAR2, V_HANDKERCHIEF, V_HEART, V_DISC,
    V_DISC2, V_WAVES, V_FAN, V_RINGS, V_SPIRAL, V_HYPERBOLIC, V_DIAMOND, V_EX,
    V_JULIA, V_EXPONENTIAL, V_POWER, V_COSINE, V_BLOB, V_PDJ, V_CYLINDER,
    V_PERSPECTIVE, V_JULIAN, V_JULIASCOPE, V_RADIAL_BLUR, V_PIE, V_NGON,
    V_CURL, V_ARCH, V_TANGENT, V_RAYS, V_BLADE, V_SECANT, V_TWINTRIAN,
    V_CROSS, V_EXP, V_LOG, V_SIN, V_COS, V_TAN, V_SEC, V_CSC, V_COT, V_SINH,
    V_COSH, V_TANH, V_SECH, V_CSCH, V_COTH, V_AUGER, V_FLUX, V_MOBIUS, V_SCRY,
    V_SPLIT, V_STRIPES, V_WEDGE, V_WEDGE_JULIA, V_WEDGE_SPH, V_WHORL,
    V_SUPERSHAPE, V_FLOWER, V_CONIC, V_PARABOLA, V_BIPOLAR, V_BOARDERS,
    V_BUTTERFLY, V_CELL, V_CPOW, V_CURVE, V_EDISC, V_ELLIPTIC, V_ESCHER,
    V_FOCI, V_LAZYSUSAN, V_LOONIE, V_OSCOPE, V_POPCORN,
    V_COUNT
};

constexpr int kFirst2D = V_SWIRL;
static_assert(V_COUNT == 98, "98 variations in the reference");

} // namespace ffr
