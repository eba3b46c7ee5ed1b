#ifndef BSV_BSV_H
#define BSV_BSV_H
/*
 * Minimal stand-in for the small-vector library "bsv" that the cvtx_ C ABI
 * is written against (include/cvortex/libcvtx.h:50 of the reference). The
 * real library is an external dependency of cvortex (CMakeLists.txt:69-71,
 * no version pin) and is not shipped with it.
 *
 * Layout contract (what the ABI depends on): bsv_V3f is a struct holding
 * exactly `float x[3]` (12 bytes), bsv_V2f holds `float x[2]` (8 bytes), the
 * double variants hold `double x[n]`. Callers index `.x[i]` and brace
 * initialise (reference test/testparticle.h:36-41).
 *
 * The helpers below are header-only conveniences with the obvious semantics
 * (component-wise arithmetic, Euclidean norm as sqrt of the left-to-right dot
 * product, exact component equality). They are inline so that this header
 * adds no symbols to any library that includes it.
 */
#include <math.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct { float x[3]; } bsv_V3f;
typedef struct { float x[2]; } bsv_V2f;
typedef struct { double x[3]; } bsv_V3d;
typedef struct { double x[2]; } bsv_V2d;

#define BSV_INLINE static inline

/* ---- 3D float ---------------------------------------------------------- */
BSV_INLINE bsv_V3f bsv_V3f_zero(void) { bsv_V3f r = {{0.f, 0.f, 0.f}}; return r; }
BSV_INLINE bsv_V3f bsv_V3f_plus(bsv_V3f a, bsv_V3f b) {
	bsv_V3f r = {{a.x[0] + b.x[0], a.x[1] + b.x[1], a.x[2] + b.x[2]}}; return r; }
BSV_INLINE bsv_V3f bsv_V3f_minus(bsv_V3f a, bsv_V3f b) {
	bsv_V3f r = {{a.x[0] - b.x[0], a.x[1] - b.x[1], a.x[2] - b.x[2]}}; return r; }
BSV_INLINE bsv_V3f bsv_V3f_mult(bsv_V3f a, float s) {
	bsv_V3f r = {{a.x[0] * s, a.x[1] * s, a.x[2] * s}}; return r; }
BSV_INLINE bsv_V3f bsv_V3f_div(bsv_V3f a, float s) {
	bsv_V3f r = {{a.x[0] / s, a.x[1] / s, a.x[2] / s}}; return r; }
BSV_INLINE float bsv_V3f_dot(bsv_V3f a, bsv_V3f b) {
	return a.x[0] * b.x[0] + a.x[1] * b.x[1] + a.x[2] * b.x[2]; }
BSV_INLINE float bsv_V3f_abs(bsv_V3f a) { return sqrtf(bsv_V3f_dot(a, a)); }
BSV_INLINE bsv_V3f bsv_V3f_cross(bsv_V3f a, bsv_V3f b) {
	bsv_V3f r = {{a.x[1] * b.x[2] - a.x[2] * b.x[1],
	              a.x[2] * b.x[0] - a.x[0] * b.x[2],
	              a.x[0] * b.x[1] - a.x[1] * b.x[0]}};
	return r; }
BSV_INLINE int bsv_V3f_isequal(bsv_V3f a, bsv_V3f b) {
	return a.x[0] == b.x[0] && a.x[1] == b.x[1] && a.x[2] == b.x[2]; }

/* ---- 2D float ---------------------------------------------------------- */
BSV_INLINE bsv_V2f bsv_V2f_zero(void) { bsv_V2f r = {{0.f, 0.f}}; return r; }
BSV_INLINE bsv_V2f bsv_V2f_plus(bsv_V2f a, bsv_V2f b) {
	bsv_V2f r = {{a.x[0] + b.x[0], a.x[1] + b.x[1]}}; return r; }
BSV_INLINE bsv_V2f bsv_V2f_minus(bsv_V2f a, bsv_V2f b) {
	bsv_V2f r = {{a.x[0] - b.x[0], a.x[1] - b.x[1]}}; return r; }
BSV_INLINE bsv_V2f bsv_V2f_mult(bsv_V2f a, float s) {
	bsv_V2f r = {{a.x[0] * s, a.x[1] * s}}; return r; }
BSV_INLINE bsv_V2f bsv_V2f_div(bsv_V2f a, float s) {
	bsv_V2f r = {{a.x[0] / s, a.x[1] / s}}; return r; }
BSV_INLINE float bsv_V2f_dot(bsv_V2f a, bsv_V2f b) {
	return a.x[0] * b.x[0] + a.x[1] * b.x[1]; }
BSV_INLINE float bsv_V2f_abs(bsv_V2f a) { return sqrtf(bsv_V2f_dot(a, a)); }
BSV_INLINE int bsv_V2f_isequal(bsv_V2f a, bsv_V2f b) {
	return a.x[0] == b.x[0] && a.x[1] == b.x[1]; }

/* ---- double helpers (used by grid redistribution code) ----------------- */
BSV_INLINE bsv_V3d bsv_V3d_zero(void) { bsv_V3d r = {{0., 0., 0.}}; return r; }
BSV_INLINE bsv_V3d bsv_V3d_plus(bsv_V3d a, bsv_V3d b) {
	bsv_V3d r = {{a.x[0] + b.x[0], a.x[1] + b.x[1], a.x[2] + b.x[2]}}; return r; }
BSV_INLINE bsv_V3d bsv_V3d_div(bsv_V3d a, double s) {
	bsv_V3d r = {{a.x[0] / s, a.x[1] / s, a.x[2] / s}}; return r; }
BSV_INLINE bsv_V3d bsv_V3f_toV3d(bsv_V3f a) {
	bsv_V3d r = {{a.x[0], a.x[1], a.x[2]}}; return r; }
BSV_INLINE bsv_V3f bsv_V3d_toV3f(bsv_V3d a) {
	bsv_V3f r = {{(float)a.x[0], (float)a.x[1], (float)a.x[2]}}; return r; }
BSV_INLINE bsv_V2d bsv_V2d_zero(void) { bsv_V2d r = {{0., 0.}}; return r; }
BSV_INLINE bsv_V2d bsv_V2d_plus(bsv_V2d a, bsv_V2d b) {
	bsv_V2d r = {{a.x[0] + b.x[0], a.x[1] + b.x[1]}}; return r; }
BSV_INLINE bsv_V2d bsv_V2d_div(bsv_V2d a, double s) {
	bsv_V2d r = {{a.x[0] / s, a.x[1] / s}}; return r; }
BSV_INLINE bsv_V2d bsv_V2f_toV2d(bsv_V2f a) {
	bsv_V2d r = {{a.x[0], a.x[1]}}; return r; }
BSV_INLINE bsv_V2f bsv_V2d_toV2f(bsv_V2d a) {
	bsv_V2f r = {{(float)a.x[0], (float)a.x[1]}}; return r; }

#undef BSV_INLINE

#ifdef __cplusplus
}
#endif
#endif /* BSV_BSV_H */
