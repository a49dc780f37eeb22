// Exact arithmetic shared by the CUDA kernels and their host-side checks.
//
// Everything here is plain binary32 / int64 arithmetic in a fixed order, so the
// same source compiled by nvcc for sm_103a (with -fmad=false) and by a host C++
// compiler (with -ffp-contract=off) gives identical bits.  These are the
// operations the reference renderer performs one pixel at a time; the GPU needs
// them in a form that any thread can evaluate for any pixel independently.
#ifndef DSRG_EXACT_H
#define DSRG_EXACT_H

#include <math.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define DSRG_HD __host__ __device__ __forceinline__
// Large helpers stay out of line on the device so that the kernels fit the instruction cache.
#define DSRG_HD_CALL static __host__ __device__ __noinline__
#else
#define DSRG_HD inline
#define DSRG_HD_CALL inline
#endif

namespace dsrg {

DSRG_HD float fadd(float a, float b) {
#if defined(__CUDA_ARCH__)
	return __fadd_rn(a, b);
#else
	return a + b;
#endif
}
DSRG_HD float fsub(float a, float b) {
#if defined(__CUDA_ARCH__)
	return __fsub_rn(a, b);
#else
	return a - b;
#endif
}
DSRG_HD float fmul(float a, float b) {
#if defined(__CUDA_ARCH__)
	return __fmul_rn(a, b);
#else
	return a * b;
#endif
}
DSRG_HD float fdiv(float a, float b) {
#if defined(__CUDA_ARCH__)
	return __fdiv_rn(a, b);
#else
	return a / b;
#endif
}
// 1 / x correctly rounded: the same value as fdiv(1.0f, x) for every x (IEEE 754 defines both as
// the rounded exact quotient), in fewer instructions on the device.
DSRG_HD float frcp(float x) {
#if defined(__CUDA_ARCH__)
	return __frcp_rn(x);
#else
	return 1.0f / x;
#endif
}
// An estimate of a / b for quotients that exact integer products correct afterwards: within 2 ulp
// on the device (|b| < 2^126, which int64 operands satisfy).  A host build may define
// DSRG_HOST_ESTIMATE_ERROR to push its estimates that far off, so that host checks exercise the
// corrections as the device does.
DSRG_HD float fdiv_estimate(float a, float b) {
#if defined(__CUDA_ARCH__)
	return __fdividef(a, b);
#elif defined(DSRG_HOST_ESTIMATE_ERROR)
	const float q = a / b;
	return q + q * DSRG_HOST_ESTIMATE_ERROR;
#else
	return a / b;
#endif
}
DSRG_HD uint32_t fbits(float f) {
#if defined(__CUDA_ARCH__)
	return __float_as_uint(f);
#else
	union { float f; uint32_t u; } v; v.f = f; return v.u;
#endif
}
DSRG_HD float bitsf(uint32_t u) {
#if defined(__CUDA_ARCH__)
	return __uint_as_float(u);
#else
	union { float f; uint32_t u; } v; v.u = u; return v.f;
#endif
}
DSRG_HD float i64_to_float(int64_t v) {
#if defined(__CUDA_ARCH__)
	return __ll2float_rn(v);
#else
	return (float)v;
#endif
}

// Result of adding d to s, n times in a row, each sum rounded to binary32 nearest-even:
//   for (i = 0; i < n; i++) s = s + d;
// The reference accumulates its depth and vertex weights this way along each
// row pair (implementation/render/shader/fillerTemplates.h:196-244, 339-372).
// Evaluated in O(binades visited) instead of O(n): inside one binade of s the
// representable values are the multiples of ulp(s), the exact sum s + d always
// has the same remainder modulo ulp(s), so every step rounds by the same
// increment until the running value leaves the binade (or a tie needs a parity
// that the current value does not have).  Those boundary steps are taken one at
// a time with a real float addition.
DSRG_HD_CALL float chain_add(float s, float d, int32_t n) {
	if (n <= 6) {
		// short chains (small triangles, quads near a row's start) are cheaper step by step
		for (int32_t i = 0; i < n; i++) s = fadd(s, d);
		return s;
	}
	for (int guard = 0; n > 0 && guard < 96; guard++) {
		uint32_t sb = fbits(s), db = fbits(d);
		int32_t se = (int32_t)((sb >> 23) & 0xFFu), de = (int32_t)((db >> 23) & 0xFFu);
		if (se == 0 || se >= 254 || de == 0 || de == 255) {
			// zero, subnormal, near-overflow, infinity or NaN: one plain step
			s = fadd(s, d); n--; continue;
		}
		const bool negative = (sb >> 31) != 0;
		const int64_t M = (int64_t)((sb & 0x7FFFFFu) | 0x800000u);     // |s| = M * 2^(se-150)
		int64_t Dm = (int64_t)((db & 0x7FFFFFu) | 0x800000u);         // |d| = Dm * 2^(de-150)
		if (((db >> 31) != 0) != negative) Dm = -Dm;                     // d relative to the sign of s
		if (de > se + 26) { s = fadd(s, d); n--; continue; }             // leaves the binade at once
		if (se > de + 26) {
			// |d| < ulp(s) / 4: s never changes unless it sits on the bottom of its binade and d
			// points down, where the next binade has a finer ulp.
			if (M == 0x800000 && Dm < 0) { s = fadd(s, d); n--; continue; }
			return s;
		}
		const int32_t e0 = se < de ? se : de;
		const int32_t ushift = se - e0;
		const int64_t U = (int64_t)1 << ushift;           // ulp(s) in units of 2^(e0-150)
		const int64_t S = M << ushift;                    // s in those units
		const int64_t D = Dm * ((int64_t)1 << (de - e0)); // d in those units
		const int64_t lo = (int64_t)1 << (23 + ushift);   // bottom of the binade of |s|
		const int64_t hi = lo << 1;
		// floor division of D by the power of two U
		int64_t a = D >> ushift;
		int64_t r = D - (a << ushift);                    // 0 <= r < U
		int64_t inc;
		if (U == 1) {
			inc = a;
		} else {
			const int64_t half = U >> 1;
			if (r < half) {
				inc = a;
			} else if (r > half) {
				inc = a + 1;
			} else {
				// tie: rounds to the even multiple; constant only once s itself is an even multiple
				if ((M & 1) != 0) { s = fadd(s, d); n--; continue; }
				inc = ((a & 1) == 0) ? a : a + 1;
			}
		}
		const int64_t X0 = S + D;
		if (X0 < lo || X0 >= hi) { s = fadd(s, d); n--; continue; }
		const int64_t INC = inc * U;
		if (INC == 0) return s;
		// m = number of steps that stay in the binade: the largest m with every k < m valid.
		// A binary32 estimate of the quotient, corrected with exact products (no 64-bit division).
		int64_t m;
		{
			const int64_t room = INC > 0 ? hi - X0 : X0 - lo; // > 0 for INC > 0, >= 0 for INC < 0
			const int64_t step = INC > 0 ? INC : -INC;
			int64_t q = (int64_t)fdiv(i64_to_float(room), i64_to_float(step));
			if (q < 0) q = 0;
			// INC > 0: count of k >= 0 with k * step < room, i.e. ceil(room / step)
			// INC < 0: count of k >= 0 with k * step <= room, i.e. floor(room / step) + 1
			if (INC > 0) {
				while (q > 0 && (q - 1) * step >= room) q--;
				while (q * step < room) q++;
			} else {
				while (q > 0 && q * step > room) q--;
				while ((q + 1) * step <= room) q++;
				q += 1;
			}
			m = q;
		}
		const int64_t steps = m < (int64_t)n ? m : (int64_t)n;
		const int64_t S2 = S + steps * INC;
		n -= (int32_t)steps;
		int64_t M2 = S2 >> (se - e0);
		uint32_t bits;
		if (M2 >= ((int64_t)1 << 24)) {
			bits = ((uint32_t)(se + 1) << 23);
		} else {
			bits = ((uint32_t)se << 23) | ((uint32_t)M2 & 0x7FFFFFu);
		}
		s = bitsf(bits | (negative ? 0x80000000u : 0u));
		if (n > 0) { s = fadd(s, d); n--; }
	}
	while (n > 0) { s = fadd(s, d); n--; }
	return s;
}

// min(max(L, (int32_t)(a / b + 1)), R) with C's truncating int64 division, as the
// reference's cutConvexEdge computes each row's bound (implementation/render/ITriangle2D.cpp:122,130).
// A binary32 estimate of the quotient settles the clamp when it is far outside
// [L, R]; near the clamp range an exact int64 remainder check corrects it; only
// quotients beyond +-2^30 (where the int32 cast may wrap) take the 64-bit division.
// Requires b != 0 and -2^20 < L <= R < 2^20.
DSRG_HD int32_t clamp_quotient_plus_one(int64_t a, int64_t b, int32_t L, int32_t R) {
	float qf = fdiv_estimate(i64_to_float(a), i64_to_float(b));
	int32_t v;
	if (qf > -1.0e9f && qf < 1.0e9f) {
		if (qf < -2097152.0f) return L;
		if (qf > 2097152.0f) return R;
		int64_t q = (int64_t)qf;
		// make the divisor positive; truncating and floor quotients are unchanged by negating both
		int64_t aa = a, bb = b;
		if (bb < 0) { aa = -aa; bb = -bb; }
		// floor quotient: q * bb <= aa < (q + 1) * bb
		while (q * bb > aa) q--;
		while ((q + 1) * bb <= aa) q++;
		if (aa < 0 && q * bb != aa) q++; // truncation toward zero
		v = (int32_t)(q + 1);
	} else {
		v = (int32_t)(a / b + 1);
	}
	return v < L ? L : (v > R ? R : v);
}

// One triangle edge in sub-pixel units, from cutConvexEdge (implementation/render/ITriangle2D.cpp:86-148).
struct Edge {
	int64_t sx, sy;      // start corner
	int64_t nx, ny;      // normal: (end.y - start.y, start.x - end.x)
	int64_t threshold;   // -1 or 0 by edge direction
};

DSRG_HD Edge make_edge(int64_t sx, int64_t sy, int64_t ex, int64_t ey) {
	Edge e;
	e.sx = sx; e.sy = sy;
	e.nx = ey - sy;
	e.ny = sx - ex;
	e.threshold = (sx > ex || (sx == ex && sy > ey)) ? -1 : 0;
	return e;
}

// Applies one edge to the interval of pixel row y, clamped to [L, R).
// The per-row limit of cutConvexEdge, limit(y) = threshold - (128 - sx)*nx - (128 + 256*y - sy)*ny,
// does not depend on the clip rectangle's corner, so any row can be cut on its own.
DSRG_HD void cut_row(const Edge &e, int32_t y, int32_t L, int32_t R, int32_t &left, int32_t &right) {
	if (e.nx != 0) {
		int64_t limit = e.threshold - (128 - e.sx) * e.nx - (128 + 256 * (int64_t)y - e.sy) * e.ny;
		int64_t offsetX = e.nx * 256;
		if (e.nx < 0) {
			int32_t side = clamp_quotient_plus_one(limit + 1, offsetX, L, R);
			if (side > left) left = side;
		} else {
			int32_t side = clamp_quotient_plus_one(limit, offsetX, L, R);
			if (side < right) right = side;
		}
	} else if (e.ny != 0) {
		int64_t value = (128 + 256 * (int64_t)y - e.sy) * e.ny;
		if (value > e.threshold) { left = R; right = L; }
	}
}

// cut_row for consecutive rows by exact integer stepping.  For a cutting edge the numerator of
// the quotient changes by the same amount every row, so the floor quotient and its remainder
// advance by a fixed quotient and remainder with at most one carry; truncation toward zero and
// the int32 wrap of (a / b + 1) then give exactly clamp_quotient_plus_one's value.  Two int64
// divisions per edge replace one division per edge and row.
struct EdgeStepper {
	int32_t kind;        // 0: cuts the left end, 1: cuts the right end, 2: empties rows (horizontal), 3: none
	int64_t q, r, B;     // floor(A / B) and A - q * B, B > 0 (A: the numerator with the divisor's sign folded in)
	int64_t qd, rd;      // the same for the change of A per row
	// horizontal edges reuse q as (128 + 256 y - sy) * ny, qd as its change per row and B as the threshold
};

// floor(a / b) and its remainder, b > 0.  Quotients below 2^22 in magnitude (every row crossing
// inside an image) come from a binary32 estimate: a and b round by at most 2^-24 relative and the
// estimated quotient by 2 ulp, so the estimate lies within 2 of a / b, and exact 64-bit products
// step its floor to the answer.  Larger quotients take the 64-bit division.
DSRG_HD void floor_divide(int64_t a, int64_t b, int64_t &q, int64_t &r) {
	const float qf = fdiv_estimate(i64_to_float(a), i64_to_float(b));
	if (qf > -4194304.0f && qf < 4194304.0f) {
		q = (int64_t)floorf(qf);
		r = a - q * b;
		while (r < 0) { q -= 1; r += b; }
		while (r >= b) { q += 1; r -= b; }
		return;
	}
	q = a / b;
	if (a % b != 0 && a < 0) q -= 1;
	r = a - q * b;
}

DSRG_HD EdgeStepper edge_stepper(const Edge &e, int32_t y0) {
	EdgeStepper s;
	s.q = s.r = s.B = s.qd = s.rd = 0;
	if (e.nx != 0) {
		int64_t a = e.threshold - (128 - e.sx) * e.nx - (128 + 256 * (int64_t)y0 - e.sy) * e.ny;
		if (e.nx < 0) a += 1;
		const int64_t b = e.nx * 256, delta = -256 * e.ny;
		const int64_t sign = b > 0 ? 1 : -1;
		s.kind = e.nx < 0 ? 0 : 1;
		s.B = b * sign;
		floor_divide(a * sign, s.B, s.q, s.r);
		floor_divide(delta * sign, s.B, s.qd, s.rd);
	} else if (e.ny != 0) {
		s.kind = 2;
		s.q = (128 + 256 * (int64_t)y0 - e.sy) * e.ny;
		s.qd = 256 * e.ny;
		s.B = e.threshold;
	} else {
		s.kind = 3;
	}
	return s;
}

// Applies the edge to the current row's interval, then moves it to the next row.
DSRG_HD void edge_step(EdgeStepper &s, int32_t L, int32_t R, int32_t &left, int32_t &right) {
	if (s.kind <= 1) {
		const int64_t t = s.q + ((s.q < 0 && s.r != 0) ? 1 : 0); // the quotient truncated toward zero
		int32_t v = (int32_t)(uint32_t)(uint64_t)(t + 1);
		v = v < L ? L : (v > R ? R : v);
		if (s.kind == 0) { if (v > left) left = v; } else { if (v < right) right = v; }
		s.q += s.qd;
		s.r += s.rd;
		if (s.r >= s.B) { s.r -= s.B; s.q += 1; }
	} else if (s.kind == 2) {
		if (s.q > s.B) { left = R; right = L; }
		s.q += s.qd;
	}
}

// Row intervals of rows [y0, y0 + rows) of a triangle, stepped (equal to row_interval of each row).
DSRG_HD void row_intervals_stepped(const int32_t *flat, int32_t y0, int32_t rows, int32_t L, int32_t R, int32_t *lefts, int32_t *rights) {
	const bool degenerate = (flat[0] == flat[2] && flat[1] == flat[3]) || (flat[2] == flat[4] && flat[3] == flat[5]) ||
	                        (flat[4] == flat[0] && flat[5] == flat[1]);
	if (degenerate) {
		for (int32_t k = 0; k < rows; k++) { lefts[k] = R; rights[k] = L; }
		return;
	}
	EdgeStepper s0 = edge_stepper(make_edge(flat[0], flat[1], flat[2], flat[3]), y0);
	EdgeStepper s1 = edge_stepper(make_edge(flat[2], flat[3], flat[4], flat[5]), y0);
	EdgeStepper s2 = edge_stepper(make_edge(flat[4], flat[5], flat[0], flat[1]), y0);
	for (int32_t k = 0; k < rows; k++) {
		int32_t left = L, right = R;
		edge_step(s0, L, R, left, right);
		edge_step(s1, L, R, left, right);
		edge_step(s2, L, R, left, right);
		lefts[k] = left;
		rights[k] = right;
	}
}

// Row interval [left, right) of pixel row y for a triangle with sub-pixel corners,
// clamped to [L, R): rasterizeTriangle (implementation/render/ITriangle2D.cpp:150-169).
DSRG_HD_CALL void row_interval(const int32_t *flat, int32_t y, int32_t L, int32_t R, int32_t &left, int32_t &right) {
	const bool degenerate = (flat[0] == flat[2] && flat[1] == flat[3]) || (flat[2] == flat[4] && flat[3] == flat[5]) ||
	                        (flat[4] == flat[0] && flat[5] == flat[1]);
	if (degenerate) { left = R; right = L; return; }
	left = L; right = R;
	for (int i = 0; i < 3; i++) {
		int j = (i + 1) % 3;
		Edge e = make_edge(flat[i * 2], flat[i * 2 + 1], flat[j * 2], flat[j * 2 + 1]);
		cut_row(e, y, L, R, left, right);
	}
}

} // namespace dsrg

#endif
