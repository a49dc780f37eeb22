// Per-fragment shading of the RgbaMultiply shader for one 2x2 quad, shared by the
// tile kernels and their host-side checks.  Integer texel mixing is exact and the
// float colour math follows the reference's operation order.
#ifndef DSRG_SHADE_H
#define DSRG_SHADE_H

#include "dsrg_exact.h"
#include "dsrg_types.h"

namespace dsrg {

DSRG_HD bool almost_zero(float v) { return v > -0.001f && v < 0.001f; } // shader/fillerTemplates.h:37-39
DSRG_HD bool almost_one(float v) { return v > 0.999f && v < 1.001f; }   // shader/fillerTemplates.h:45-47
DSRG_HD bool almost_same3(const float *c) {                             // shader/fillerTemplates.h:53-55
	return almost_zero(c[0] - c[1]) && almost_zero(c[0] - c[2]) && almost_zero(c[1] - c[2]);
}
DSRG_HD bool almost_one3(const float *c) { return almost_one(c[0]) && almost_one(c[1]) && almost_one(c[2]); }

// truncateToU32 of the reference's scalar build: a signed 64-bit truncation keeping the low 32 bits.
DSRG_HD uint32_t trunc_u32(float x) {
	if (!(x == x)) return 0u;
	if (x >= 9.2233720368547758e18f || x <= -9.2233720368547758e18f) return 0u;
	return (uint32_t)(int64_t)x;
}

// (a*wa + b*wb) >> 8 per byte channel: weightColors (api/textureAPI.h:242-255).
DSRG_HD uint32_t weight_colors(uint32_t a, uint32_t wa, uint32_t b, uint32_t wb) {
	uint32_t low = (((a & 0x00FF00FFu) * wa + (b & 0x00FF00FFu) * wb) >> 8) & 0x00FF00FFu;
	uint32_t high = ((((a >> 8) & 0x00FF00FFu) * wa + ((b >> 8) & 0x00FF00FFu) * wb)) & 0xFF00FF00u;
	return low | high;
}

// texture_interpolate_color_bilinear (api/textureAPI.h:310-318).
DSRG_HD uint32_t bilinear_mix(uint32_t a, uint32_t b, uint32_t c, uint32_t d, uint32_t wx, uint32_t wy) {
	return weight_colors(weight_colors(a, 256u - wx, b, wx), 256u - wy, weight_colors(c, 256u - wx, d, wx), wy);
}

DSRG_HD uint32_t texel_load(const uint32_t *p, uint32_t index) {
#if defined(__CUDA_ARCH__)
	return __ldg(p + index);
#else
	return p[index];
#endif
}

// texture_sample_bilinear with MIP_INSIDE (api/textureAPI.h:320-430).
DSRG_HD uint32_t sample_bilinear(const TextureData &t, float u, float v, uint32_t mip, bool highest) {
	uint32_t scaleU = 256u << t.log2width, scaleV = 256u << t.log2height;
	uint32_t maskX = t.maxWidthAndMask, maskY = t.maxHeightAndMask;
	uint32_t log2Stride = t.log2width;
	uint32_t layer = t.startOffset;
	if (!highest) {
		scaleU >>= mip; scaleV >>= mip; maskX >>= mip; maskY >>= mip;
		log2Stride -= mip;
		layer = t.startOffset & (t.maxLevelMask >> (mip << 1));
	}
	uint32_t sx = trunc_u32(fmul(fadd(u, 256.0f), (float)scaleU)) - 128u;
	uint32_t sy = trunc_u32(fmul(fadd(v, 256.0f), (float)scaleV)) - 128u;
	uint32_t wx = sx & 0xFFu, wy = sy & 0xFFu;
	uint32_t left = sx >> 8, top = sy >> 8;
	uint32_t right = (left + 1u) & maskX, bottom = (top + 1u) & maskY;
	left &= maskX; top &= maskY;
	uint32_t upper = top << log2Stride, lower = bottom << log2Stride;
	uint32_t a = texel_load(t.pixels, (upper | left) + layer);
	uint32_t b = texel_load(t.pixels, (upper | right) + layer);
	uint32_t c = texel_load(t.pixels, (lower | left) + layer);
	uint32_t d = texel_load(t.pixels, (lower | right) + layer);
	return bilinear_mix(a, b, c, d, wx, wy);
}

DSRG_HD float fabs_exact(float v) { return bitsf(fbits(v) & 0x7FFFFFFFu); }
DSRG_HD float fmax_ref(float a, float b) { return (a > b) ? a : b; } // base/noSimd.h:145-147

// texture_getMipLevelIndex (api/textureAPI.h:471-495) from lanes 0 (upper left), 1 (upper right), 2 (lower left).
DSRG_HD uint32_t mip_level(const TextureData &t, const float *u, const float *v) {
	float offsetU = fmul(fmax_ref(fabs_exact(u[0] - u[1]), fabs_exact(u[0] - u[2])), t.floatMaxWidth);
	float offsetV = fmul(fmax_ref(fabs_exact(v[0] - v[1]), fabs_exact(v[0] - v[2])), t.floatMaxHeight);
	float offset = fmax_ref(offsetU, offsetV);
	int32_t result = 0;
	if (offset > 2.0f) result = 1;
	if (offset > 4.0f) result = 2;
	if (offset > 8.0f) result = 3;
	if (offset > 16.0f) result = 4;
	if (result > (int32_t)t.maxMipLevel) result = (int32_t)t.maxMipLevel;
	return (uint32_t)result;
}

// shaderMethods::interpolate (shader/shaderMethods.h:39-45).
DSRG_HD float interpolate3(const float *v, float wa, float wb, float wc) {
	return fadd(fadd(fmul(v[0], wa), fmul(v[1], wb)), fmul(v[2], wc));
}

DSRG_HD void unpack_rgba(uint32_t c, float *out) {
	out[0] = (float)(c & 0xFFu); out[1] = (float)((c >> 8) & 0xFFu);
	out[2] = (float)((c >> 16) & 0xFFu); out[3] = (float)(c >> 24);
}

// getPixels_2x2 (shader/RgbaMultiply.h:74-106) for lane `lane` of a quad whose four lanes have
// vertex weights wa/wb/wc.  The mip level of each texture comes from lanes 0..2.
// a[lane] by selects, so that arrays indexed by a run-time lane stay in registers
DSRG_HD float pick4(const float *a, int lane) { return lane == 0 ? a[0] : (lane == 1 ? a[1] : (lane == 2 ? a[2] : a[3])); }

DSRG_HD void shade_lane_inline(const ShadeRecord &s, const TextureData *textures, const float *wa, const float *wb,
                               const float *wc, int lane, float *rgba) {
	const bool hasDiffuse = (s.flags & SHADE_DIFFUSE) != 0, hasLight = (s.flags & SHADE_LIGHT) != 0;
	const bool colorless = (s.flags & SHADE_COLORLESS) != 0, fade = (s.flags & SHADE_VERTEX_FADE) != 0;
	float u[4], v[4];
	if (hasDiffuse && !hasLight && colorless) {
		const TextureData &t = textures[s.diffuse];
		for (int l = 0; l < 3; l++) { u[l] = interpolate3(s.u1, wa[l], wb[l], wc[l]); v[l] = interpolate3(s.v1, wa[l], wb[l], wc[l]); }
		u[3] = interpolate3(s.u1, wa[3], wb[3], wc[3]); v[3] = interpolate3(s.v1, wa[3], wb[3], wc[3]);
		unpack_rgba(sample_bilinear(t, pick4(u, lane), pick4(v, lane), mip_level(t, u, v), false), rgba);
		return;
	}
	if (hasLight && !hasDiffuse && colorless) {
		const TextureData &t = textures[s.light];
		float uu = interpolate3(s.u2, pick4(wa, lane), pick4(wb, lane), pick4(wc, lane)), vv = interpolate3(s.v2, pick4(wa, lane), pick4(wb, lane), pick4(wc, lane));
		unpack_rgba(sample_bilinear(t, uu, vv, 0u, true), rgba);
		return;
	}
	if (fade) {
		rgba[0] = interpolate3(s.red, pick4(wa, lane), pick4(wb, lane), pick4(wc, lane));
		rgba[1] = interpolate3(s.green, pick4(wa, lane), pick4(wb, lane), pick4(wc, lane));
		rgba[2] = interpolate3(s.blue, pick4(wa, lane), pick4(wb, lane), pick4(wc, lane));
		rgba[3] = interpolate3(s.alpha, pick4(wa, lane), pick4(wb, lane), pick4(wc, lane));
	} else {
		rgba[0] = s.red[0]; rgba[1] = s.green[0]; rgba[2] = s.blue[0]; rgba[3] = s.alpha[0];
	}
	float texel[4];
	if (hasDiffuse) {
		const TextureData &t = textures[s.diffuse];
		for (int l = 0; l < 4; l++) { u[l] = interpolate3(s.u1, wa[l], wb[l], wc[l]); v[l] = interpolate3(s.v1, wa[l], wb[l], wc[l]); }
		unpack_rgba(sample_bilinear(t, pick4(u, lane), pick4(v, lane), mip_level(t, u, v), false), texel);
		for (int ch = 0; ch < 4; ch++) rgba[ch] = fmul(rgba[ch], texel[ch]);
	}
	if (hasLight) {
		const TextureData &t = textures[s.light];
		float uu = interpolate3(s.u2, pick4(wa, lane), pick4(wb, lane), pick4(wc, lane)), vv = interpolate3(s.v2, pick4(wa, lane), pick4(wb, lane), pick4(wc, lane));
		unpack_rgba(sample_bilinear(t, uu, vv, 0u, true), texel);
		for (int ch = 0; ch < 4; ch++) rgba[ch] = fmul(rgba[ch], texel[ch]);
	}
}

// shade_lane_inline kept out of line, for kernels where its code size matters more than keeping
// its inputs in registers.
DSRG_HD_CALL void shade_lane(const ShadeRecord &s, const TextureData *textures, const float *wa, const float *wb,
                             const float *wc, int lane, float *rgba) {
	shade_lane_inline(s, textures, wa, wb, wc, lane, rgba);
}


// shade_lane for every lane of `mask` at once: the texture coordinates of the quad's four lanes
// and the mip levels are evaluated once and shared, each covered lane then samples on its own.
// rgba[lane] is written for the lanes of the mask, with the same values shade_lane gives.
// One lane of shade_quad, given the quad's diffuse coordinates u, v and mip level (computed once
// for the quad when the diffuse map exists); in line, so that a caller that unrolls the lanes keeps
// every array in registers.
DSRG_HD void shade_quad_lane(const ShadeRecord &s, const TextureData *textures, const float *wa, const float *wb, const float *wc,
                             const float *u, const float *v, uint32_t diffuseMip, int lane, float *out) {
	const bool hasDiffuse = (s.flags & SHADE_DIFFUSE) != 0, hasLight = (s.flags & SHADE_LIGHT) != 0;
	const bool colorless = (s.flags & SHADE_COLORLESS) != 0, fade = (s.flags & SHADE_VERTEX_FADE) != 0;
	if (hasDiffuse && !hasLight && colorless) {
		unpack_rgba(sample_bilinear(textures[s.diffuse], u[lane], v[lane], diffuseMip, false), out);
		return;
	}
	if (hasLight && !hasDiffuse && colorless) {
		const float uu = interpolate3(s.u2, wa[lane], wb[lane], wc[lane]), vv = interpolate3(s.v2, wa[lane], wb[lane], wc[lane]);
		unpack_rgba(sample_bilinear(textures[s.light], uu, vv, 0u, true), out);
		return;
	}
	if (fade) {
		out[0] = interpolate3(s.red, wa[lane], wb[lane], wc[lane]);
		out[1] = interpolate3(s.green, wa[lane], wb[lane], wc[lane]);
		out[2] = interpolate3(s.blue, wa[lane], wb[lane], wc[lane]);
		out[3] = interpolate3(s.alpha, wa[lane], wb[lane], wc[lane]);
	} else {
		out[0] = s.red[0]; out[1] = s.green[0]; out[2] = s.blue[0]; out[3] = s.alpha[0];
	}
	float texel[4];
	if (hasDiffuse) {
		unpack_rgba(sample_bilinear(textures[s.diffuse], u[lane], v[lane], diffuseMip, false), texel);
		for (int ch = 0; ch < 4; ch++) out[ch] = fmul(out[ch], texel[ch]);
	}
	if (hasLight) {
		const float uu = interpolate3(s.u2, wa[lane], wb[lane], wc[lane]), vv = interpolate3(s.v2, wa[lane], wb[lane], wc[lane]);
		unpack_rgba(sample_bilinear(textures[s.light], uu, vv, 0u, true), texel);
		for (int ch = 0; ch < 4; ch++) out[ch] = fmul(out[ch], texel[ch]);
	}
}

// The diffuse coordinates and mip level of a quad (lanes 0..2 choose the level).
DSRG_HD uint32_t quad_diffuse_coordinates(const ShadeRecord &s, const TextureData *textures, const float *wa, const float *wb,
                                          const float *wc, float *u, float *v) {
	if ((s.flags & SHADE_DIFFUSE) == 0) return 0;
	for (int l = 0; l < 4; l++) { u[l] = interpolate3(s.u1, wa[l], wb[l], wc[l]); v[l] = interpolate3(s.v1, wa[l], wb[l], wc[l]); }
	return mip_level(textures[s.diffuse], u, v);
}

// Byte index of red, green, blue, alpha for PackOrderIndex RGBA, BGRA, ARGB, ABGR (image/PackOrder.h:80-92).
DSRG_HD uint32_t pack_shift(int32_t packOrder, int ch) {
	switch (packOrder) {
		case 1: { const uint32_t s[4] = {16u, 8u, 0u, 24u}; return s[ch]; }
		case 2: { const uint32_t s[4] = {8u, 16u, 24u, 0u}; return s[ch]; }
		case 3: { const uint32_t s[4] = {24u, 16u, 8u, 0u}; return s[ch]; }
		default: { const uint32_t s[4] = {0u, 8u, 16u, 24u}; return s[ch]; }
	}
}

// packOrder_floatToSaturatedByte with an order (image/PackOrder.h:204-212).
DSRG_HD uint32_t pack_saturated(const float *rgba, int32_t packOrder) {
	uint32_t out = 0;
	for (int ch = 0; ch < 4; ch++) {
		float c = rgba[ch];
		float clamped = (255.1f < c) ? 255.1f : c;
		out |= trunc_u32(clamped) << pack_shift(packOrder, ch);
	}
	return out;
}

} // namespace dsrg

#endif
