// Device pieces shared by the tile kernels and the differentiable renderer: the reference's
// row-pair bounds and running sums for one quad, the vertex weights of a fragment, and the
// 64-bit depth keys.
#ifndef DSRG_RASTER_CUH
#define DSRG_RASTER_CUH

#include "dsrg_exact.h"
#include "dsrg_types.h"

namespace dsrg {

// Largest k in [0, count) with base[k] <= i (base[0] = 0, ascending).
__device__ __forceinline__ int32_t find_segment(const uint32_t *base, int32_t count, uint32_t i) {
	int32_t lo = 0, hi = count - 1;
	while (lo < hi) {
		const int32_t mid = (lo + hi + 1) >> 1;
		if (__ldg(&base[mid]) <= i) lo = mid; else hi = mid - 1;
	}
	return lo;
}

// find_segment over a copy of the bases in shared memory.
__device__ __forceinline__ int32_t find_segment_shared(const uint32_t *base, int32_t count, uint32_t i) {
	int32_t lo = 0, hi = count - 1;
	while (lo < hi) {
		const int32_t mid = (lo + hi + 1) >> 1;
		if (base[mid] <= i) lo = mid; else hi = mid - 1;
	}
	return lo;
}

__device__ __forceinline__ void unpack_row(uint32_t packed, int32_t &left, int32_t &right) {
	left = (int32_t)(packed & 0xFFFFu);
	right = (int32_t)(packed >> 16);
}

// Block bounds of one row pair (fillerTemplates.h:273-293).
struct RowPair {
	int32_t obs, obe, ibs, ibe;
	int32_t upperLeft, upperRight, lowerLeft, lowerRight;
	bool any;
};

__device__ __forceinline__ RowPair make_row_pair(int32_t uL, int32_t uR, int32_t lL, int32_t lR, int32_t y2, int32_t maxHeight) {
	RowPair rp;
	int32_t outerStart = min(uL, lL), outerEnd = max(uR, lR);
	int32_t innerStart = max(uL, lL), innerEnd = min(uR, lR);
	rp.obs = (int32_t)((uint32_t)outerStart & ~1u);
	rp.obe = (int32_t)(((uint32_t)outerEnd + 1u) & ~1u);
	rp.ibs = (int32_t)(((uint32_t)innerStart + 1u) & ~1u);
	rp.ibe = (int32_t)((uint32_t)innerEnd & ~1u);
	if (y2 >= maxHeight) lR = lL;
	rp.upperLeft = uL; rp.upperRight = uR; rp.lowerLeft = lL; rp.lowerRight = lR;
	rp.any = (uR > uL) || (lR > lL);
	return rp;
}

// Row pair of a record for the rows y1, y1 + 1 from its row intervals (recordRows = its first row;
// row offsets are even because raster bounds are row-pair aligned, so two rows load as one uint2).
__device__ __forceinline__ RowPair record_row_pair(const DrawRecord &r, const uint32_t *recordRows, int32_t y1, int32_t height) {
	int32_t uL, uR, lL, lR;
	const uint2 two = *reinterpret_cast<const uint2 *>(recordRows + (y1 - r.top));
	unpack_row(two.x, uL, uR);
	unpack_row(two.y, lL, lR);
	return make_row_pair(uL, uR, lL, lR, y1 + 1, height);
}

// chain_add for the short chains of small triangles: up to three additions straight in line
// (predicated, no loop and no call), longer chains through chain_add.
__device__ __forceinline__ float chain_add_short(float s, float d, int32_t n) {
	if (n <= 3) {
		if (n > 0) s = fadd(s, d);
		if (n > 1) s = fadd(s, d);
		if (n > 2) s = fadd(s, d);
		return s;
	}
	return chain_add(s, d, n);
}

// The four lane values of one component (1/W or W, U/W, V/W) for the quad at x, following the
// reference's accumulation: edge quads step pWeightUpper/Lower by 2*dx one quad at a time, the
// run of full quads steps every lane on its own from where the left edge stopped, and the right
// edge restarts from the left edge's value plus 2*dx times the run length
// (fillerTemplates.h:196-244, 328-373).
__device__ __forceinline__ void quad_lanes(float start, float dx, float dy, const RowPair &rp, int32_t y1, int32_t x, float *out) {
	const float P0 = fadd(fadd(start, fmul(dx, (float)rp.obs + 0.5f)), fmul(dy, (float)y1 + 0.5f));
	const float L0 = fadd(P0, dy);
	const float d2 = fmul(dx, 2.0f);
	if (rp.ibe <= rp.ibs || x < rp.ibs) {
		int32_t k = (x - rp.obs) >> 1;
		float U = chain_add_short(P0, d2, k), L = chain_add_short(L0, d2, k);
		out[0] = U; out[1] = fadd(U, dx); out[2] = L; out[3] = fadd(L, dx);
		return;
	}
	const int32_t nL = (rp.ibs - rp.obs) >> 1;
	const float Ub = chain_add_short(P0, d2, nL), Lb = chain_add_short(L0, d2, nL);
	if (x < rp.ibe) {
		int32_t j = (x - rp.ibs) >> 1;
		out[0] = chain_add_short(Ub, d2, j);
		out[1] = chain_add_short(fadd(Ub, dx), d2, j);
		out[2] = chain_add_short(Lb, d2, j);
		out[3] = chain_add_short(fadd(Lb, dx), d2, j);
	} else {
		int32_t nI = (rp.ibe - rp.ibs) >> 1, r = (x - rp.ibe) >> 1;
		float m = fmul(d2, (float)nI);
		float U = chain_add_short(fadd(Ub, m), d2, r), L = chain_add_short(fadd(Lb, m), d2, r);
		out[0] = U; out[1] = fadd(U, dx); out[2] = L; out[3] = fadd(L, dx);
	}
}

// Position `lane` of quad_lanes alone: the same operations on the same values, for the one chain
// that position's value comes from.
__device__ __forceinline__ float quad_lane(float start, float dx, float dy, const RowPair &rp, int32_t y1, int32_t x, int lane) {
	const float P0 = fadd(fadd(start, fmul(dx, (float)rp.obs + 0.5f)), fmul(dy, (float)y1 + 0.5f));
	const float R0 = (lane < 2) ? P0 : fadd(P0, dy);
	const float d2 = fmul(dx, 2.0f);
	const bool odd = (lane & 1) != 0;
	if (rp.ibe <= rp.ibs || x < rp.ibs) {
		const float v = chain_add_short(R0, d2, (x - rp.obs) >> 1);
		return odd ? fadd(v, dx) : v;
	}
	const float B = chain_add_short(R0, d2, (rp.ibs - rp.obs) >> 1);
	if (x < rp.ibe) return chain_add_short(odd ? fadd(B, dx) : B, d2, (x - rp.ibs) >> 1);
	const float m = fmul(d2, (float)((rp.ibe - rp.ibs) >> 1));
	const float v = chain_add_short(fadd(B, m), d2, (x - rp.ibe) >> 1);
	return odd ? fadd(v, dx) : v;
}

// Whether the quad at x lies in the pair's run of full quads (fillerTemplates.h:357-364).
__device__ __forceinline__ bool full_quad(const RowPair &rp, int32_t x) {
	return rp.ibe > rp.ibs && x >= rp.ibs && x < rp.ibe;
}

// The last row of a target of odd height.  Its row pair's lower row lies outside the image: the
// reference empties that row's interval but bounds the run of full quads with the row as it was,
// and points the lower row's pixels at the upper row (fillerTemplates.h:285-306).  In that run the
// lower lanes are therefore tested against and written into the upper row, after the upper lanes.
__device__ __forceinline__ bool odd_last_row(int32_t py, int32_t height) {
	return (height & 1) != 0 && py == height - 1;
}

// Whether lane l of the quad at x is drawn (clipPixels, fillerTemplates.h:92-106); full quads draw all four.
__device__ __forceinline__ bool lane_covered(const RowPair &rp, int32_t x, bool edge, int l) {
	if (!edge) return true;
	const int32_t xx = x + (l & 1);
	return (l < 2) ? (xx >= rp.upperLeft && xx < rp.upperRight) : (xx >= rp.lowerLeft && xx < rp.lowerRight);
}

__device__ __forceinline__ uint32_t ordered_depth(float z) {
	uint32_t bits = fbits(z);
	if (bits == 0x80000000u) bits = 0u; // -0 and +0 compare equal
	return (bits & 0x80000000u) ? ~bits : (bits | 0x80000000u);
}

__device__ __forceinline__ unsigned long long make_key(float z, uint32_t record, bool depthTest, bool affine) {
	if (!depthTest) return (unsigned long long)(record + 1u); // no depth buffer: the last triangle drawn wins
	uint32_t hi = ordered_depth(z);
	if (affine) hi = ~hi;
	return ((unsigned long long)hi << 32) | (unsigned long long)(~record);
}

__device__ __forceinline__ uint32_t key_record(unsigned long long key, bool depthTest) {
	return depthTest ? ~(uint32_t)(key & 0xFFFFFFFFull) : (uint32_t)key - 1u;
}

// Vertex weights of one position from its (1/W, U/W, V/W) or (W, U, V), as lane_weights gives them.
__device__ __forceinline__ void lane_weight(float w0, float w1, float w2, bool affine, float &wa, float &wb, float &wc) {
	if (affine) {
		wb = w1;
		wc = w2;
	} else {
		const float linearDepth = frcp(w0); // reciprocal of the scalar build (noSimd.h:187)
		wb = fmul(w1, linearDepth);
		wc = fmul(w2, linearDepth);
	}
	wa = 1.0f - fadd(wb, wc);
}

// Vertex weights of the four lanes from (1/W, U/W, V/W) or (W, U, V) (fillerTemplates.h:197-233).
__device__ __forceinline__ void lane_weights(const float (*w)[4], bool affine, float *wa, float *wb, float *wc) {
	for (int l = 0; l < 4; l++) {
		if (affine) {
			wb[l] = w[1][l];
			wc[l] = w[2][l];
		} else {
			const float linearDepth = frcp(w[0][l]); // reciprocal of the scalar build (noSimd.h:187)
			wb[l] = fmul(w[1][l], linearDepth);
			wc[l] = fmul(w[2][l], linearDepth);
		}
		wa[l] = 1.0f - fadd(wb[l], wc[l]);
	}
}

} // namespace dsrg

#endif
