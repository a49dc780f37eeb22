// Host build of the exact arithmetic that the kernels use (dsrg_exact.h, dsrg_geometry.h),
// exported for CPU-side checks of the closed-form accumulation and the row intervals.
// Built with -ffp-contract=off so that it computes the same bits as the device code.
#include <stdint.h>

// Estimates of integer quotients 2^-21 off, at least as far as the device's: the host checks then
// exercise the exact corrections that follow them.
#define DSRG_HOST_ESTIMATE_ERROR 4.76837158203125e-7f
#include "dsrg_exact.h"
#include "dsrg_geometry.h"

extern "C" {

// out[i] = s[i] after n[i] additions of d[i] (dsrg::chain_add).
void dsrg_host_chain_add(const float *s, const float *d, const int32_t *n, float *out, int64_t count) {
	for (int64_t i = 0; i < count; i++) out[i] = dsrg::chain_add(s[i], d[i], n[i]);
}

// out[i] = min(max(L, (int32)(a/b + 1)), R) (dsrg::clamp_quotient_plus_one).
void dsrg_host_clamp_quotient(const int64_t *a, const int64_t *b, const int32_t *L, const int32_t *R, int32_t *out, int64_t count) {
	for (int64_t i = 0; i < count; i++) out[i] = dsrg::clamp_quotient_plus_one(a[i], b[i], L[i], R[i]);
}

// Row intervals of one triangle (sub-pixel corners flat[6]) for rows [y0, y0 + rows), clamped to [L, R).
void dsrg_host_row_intervals(const int32_t *flat, int32_t y0, int32_t rows, int32_t L, int32_t R, int32_t *lefts, int32_t *rights) {
	for (int32_t r = 0; r < rows; r++) dsrg::row_interval(flat, y0 + r, L, R, lefts[r], rights[r]);
}

// The same rows by exact stepping (dsrg::row_intervals_stepped).
void dsrg_host_row_intervals_stepped(const int32_t *flat, int32_t y0, int32_t rows, int32_t L, int32_t R, int32_t *lefts,
                                     int32_t *rights) {
	dsrg::row_intervals_stepped(flat, y0, rows, L, R, lefts, rights);
}

} // extern "C"
