/*
 * CPU oracle for the DFPSR triangle-rendering hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * Scalar restatement of the reference's model_render / renderer_* / model_renderDepth
 * path in plain C.  Used only by tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg as the checker.  Build with -ffp-contract=off.
 *
 * File:line citations are relative to the reference's Source/ directory.
 */
#include "dsr_oracle.h"

#include <math.h>
#include <float.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define UNITS_PER_PIXEL 256      /* DFPSR/implementation/render/constants.h:39 */
#define UNITS_PER_HALF_PIXEL 128 /* constants.h:40 */

typedef struct { float x, y, z; } v3;
typedef struct { float x, y; } v2;
typedef struct { int64_t x, y; } l2;
typedef struct { v3 cs; v2 is; l2 flat; } projected;          /* ProjectedPoint.h:33-49 */
typedef struct { v3 normal; float offset; } plane3;          /* math/FPlane3D.h:30-46 */
typedef struct { int32_t left, top, right, bottom; } irect;  /* math/IRect.h (stored as bounds) */
typedef struct { int32_t left, right; } row_interval;        /* ITriangle2D.h:37-44 */

static inline v3 mk3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 add3(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 scale3(v3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
static inline float dot3(v3 a, v3 b) { return (a.x * b.x) + (a.y * b.y) + (a.z * b.z); } /* math/FVector.h:74-76 */

static inline int32_t imin(int32_t a, int32_t b) { return (a < b) ? a : b; } /* base/noSimd.h:134-136 */
static inline int32_t imax(int32_t a, int32_t b) { return (a > b) ? a : b; } /* base/noSimd.h:145-147 */
static inline float fmaxf_ref(float a, float b) { return (a > b) ? a : b; }

/* truncateToU32 of the scalar build (base/simd.h:2726-2732 scalar branch): gcc on x86-64
 * converts through a signed 64-bit truncation and keeps the low 32 bits. */
static inline uint32_t trunc_u32(float x) {
	if (x != x) return 0u;
	if (x >= 9.2233720368547758e18f || x <= -9.2233720368547758e18f) return 0u;
	return (uint32_t)(int64_t)x;
}

/* ------------------------------------------------------------------ camera */

/* FPlane3D(normal, offset) normalizes its normal (math/FPlane3D.h:36, FVector.h:113-119). */
static plane3 make_plane(float x, float y, float z, float offset) {
	plane3 p;
	float l = sqrtf(x * x + y * y + z * z);
	if (l == 0.0f) {
		p.normal = mk3(0.0f, 0.0f, 1.0f);
	} else {
		p.normal = mk3(x / l, y / l, z / l);
	}
	p.offset = offset;
	return p;
}

static inline int plane_inside(const plane3 *p, v3 point) { /* FPlane3D.h:41-46 */
	return (dot3(p->normal, point) - p->offset) <= 0.0f;
}

typedef struct {
	int perspective;
	v3 position, xAxis, yAxis, zAxis;
	float widthSlope, heightSlope, invWidthSlope, invHeightSlope, imageWidth, imageHeight, nearClip, farClip;
	int cullCount, clipCount;
	plane3 cull[6], clip[6];
} camera;

/* ViewFrustum constructors (implementation/render/Camera.h:55-74). */
static int frustum_perspective(plane3 *planes, float nearClip, float farClip, float ws, float hs) {
	planes[0] = make_plane(-1.0f, 0.0f, -ws, 0.0f);
	planes[1] = make_plane(1.0f, 0.0f, -ws, 0.0f);
	planes[2] = make_plane(0.0f, 1.0f, -hs, 0.0f);
	planes[3] = make_plane(0.0f, -1.0f, -hs, 0.0f);
	planes[4] = make_plane(0.0f, 0.0f, -1.0f, -nearClip);
	planes[5] = make_plane(0.0f, 0.0f, 1.0f, farClip);
	return (farClip == INFINITY) ? 5 : 6;
}
static int frustum_orthogonal(plane3 *planes, float halfWidth, float halfHeight) {
	planes[0] = make_plane(-1.0f, 0.0f, 0.0f, halfWidth);
	planes[1] = make_plane(1.0f, 0.0f, 0.0f, halfWidth);
	planes[2] = make_plane(0.0f, 1.0f, 0.0f, halfHeight);
	planes[3] = make_plane(0.0f, -1.0f, 0.0f, halfHeight);
	return 4;
}

/* Camera::createPerspective / createOrthogonal (Camera.h:139-156). */
static void camera_create(camera *c, const or_camera_desc *d) {
	const float *t = d->location;
	c->position = mk3(t[0], t[1], t[2]);
	c->xAxis = mk3(t[3], t[4], t[5]);
	c->yAxis = mk3(t[6], t[7], t[8]);
	c->zAxis = mk3(t[9], t[10], t[11]);
	c->imageWidth = (float)d->width;
	c->imageHeight = (float)d->height;
	c->perspective = d->perspective;
	if (d->perspective) {
		float ws = d->slope;
		float hs = ws * c->imageHeight / c->imageWidth;
		c->widthSlope = ws; c->heightSlope = hs;
		c->nearClip = d->nearClip; c->farClip = d->farClip;
		c->cullCount = frustum_perspective(c->cull, d->nearClip, d->farClip, ws * 1.0001f, hs * 1.0001f);
		c->clipCount = frustum_perspective(c->clip, d->nearClip, d->farClip, ws * 2.0f, hs * 2.0f);
	} else {
		float hw = d->slope;
		float hh = hw * c->imageHeight / c->imageWidth;
		c->widthSlope = hw; c->heightSlope = hh;
		c->nearClip = -FLT_MAX; c->farClip = INFINITY;
		c->cullCount = frustum_orthogonal(c->cull, hw * 1.0001f, hh * 1.0001f);
		c->clipCount = frustum_orthogonal(c->clip, hw * 2.0f, hh * 2.0f);
	}
	c->invWidthSlope = 0.5f / c->widthSlope;
	c->invHeightSlope = 0.5f / c->heightSlope;
}

/* Transform3D::transformPoint (math/Transform3D.h:39-41, FMatrix3x3.h:55-61). */
static v3 transform_point(const float *m, v3 p) {
	v3 r;
	r.x = p.x * m[3] + p.y * m[6] + p.z * m[9];
	r.y = p.x * m[4] + p.y * m[7] + p.z * m[10];
	r.z = p.x * m[5] + p.y * m[8] + p.z * m[11];
	return add3(r, mk3(m[0], m[1], m[2]));
}

/* Camera::worldToCamera = transformPointTransposedInverse (Camera.h:157-159, Transform3D.h:49-51,
 * FMatrix3x3.h:66-72). */
static v3 world_to_camera(const camera *c, v3 p) {
	v3 d = sub3(p, c->position);
	return mk3(d.x * c->xAxis.x + d.y * c->xAxis.y + d.z * c->xAxis.z,
	           d.x * c->yAxis.x + d.y * c->yAxis.y + d.z * c->yAxis.z,
	           d.x * c->zAxis.x + d.y * c->zAxis.y + d.z * c->zAxis.z);
}

/* Camera::cameraToScreen (Camera.h:160-187). */
static projected camera_to_screen(const camera *c, v3 cs) {
	projected p;
	p.cs = cs;
	if (c->perspective) {
		float invDepth = (cs.z > 0.0f) ? 1.0f / cs.z : 0.0f;
		float centerShear = cs.z * 0.5f;
		float preX = (cs.x * c->invWidthSlope + centerShear) * c->imageWidth;
		float preY = (-cs.y * c->invHeightSlope + centerShear) * c->imageHeight;
		p.is.x = preX * invDepth;
		p.is.y = preY * invDepth;
	} else {
		p.is.x = (cs.x * c->invWidthSlope + 0.5f) * c->imageWidth;
		p.is.y = (-cs.y * c->invHeightSlope + 0.5f) * c->imageHeight;
	}
	float subX = p.is.x * (float)UNITS_PER_PIXEL;
	float subY = p.is.y * (float)UNITS_PER_PIXEL;
	p.flat.x = (int64_t)subX;
	p.flat.y = (int64_t)subY;
	return p;
}

void or_camera_to_screen(const or_camera_desc *desc, const float cs[3], float outIs[2], int64_t outFlat[2]) {
	camera c;
	camera_create(&c, desc);
	projected p = camera_to_screen(&c, mk3(cs[0], cs[1], cs[2]));
	outIs[0] = p.is.x; outIs[1] = p.is.y;
	outFlat[0] = p.flat.x; outFlat[1] = p.flat.y;
}

/* Camera::worldToScreen (Camera.h:188-190): out = cs.x, cs.y, cs.z, is.x, is.y; outFlat = flat. */
void or_world_to_screen(const or_camera_desc *desc, const float world[3], float out[5], int64_t outFlat[2]) {
	camera c;
	camera_create(&c, desc);
	projected p = camera_to_screen(&c, world_to_camera(&c, mk3(world[0], world[1], world[2])));
	out[0] = p.cs.x; out[1] = p.cs.y; out[2] = p.cs.z; out[3] = p.is.x; out[4] = p.is.y;
	outFlat[0] = p.flat.x; outFlat[1] = p.flat.y;
}

/* ViewFrustum::isConvexHullSeen (Camera.h:87-108). */
static int convex_hull_seen(const plane3 *planes, int planeCount, const v3 *points, int count) {
	int anyOutside = 0;
	for (int s = 0; s < planeCount; s++) {
		int anyInside = 0;
		for (int p = 0; p < count; p++) {
			if (plane_inside(&planes[s], points[p])) anyInside = 1; else anyOutside = 1;
		}
		if (!anyInside) return 0;
	}
	return anyOutside ? 1 : 2;
}

/* Camera::isBoxSeen (Camera.h:202-217). */
static int box_seen(const camera *c, v3 mn, v3 mx, const float *modelToWorld) {
	v3 corners[8];
	v3 local[8] = {
		{mn.x, mn.y, mn.z}, {mx.x, mn.y, mn.z}, {mn.x, mx.y, mn.z}, {mx.x, mx.y, mn.z},
		{mn.x, mn.y, mx.z}, {mx.x, mn.y, mx.z}, {mn.x, mx.y, mx.z}, {mx.x, mx.y, mx.z}};
	for (int i = 0; i < 8; i++) corners[i] = world_to_camera(c, transform_point(modelToWorld, local[i]));
	return convex_hull_seen(c->cull, c->cullCount, corners, 8);
}

/* ------------------------------------------------------------------ ITriangle2D */

typedef struct {
	projected position[3];
	irect wholeBound;
} triangle2d;

/* getTriangleBound (implementation/render/ITriangle2D.cpp:31-43); int64 truncating division. */
static irect triangle_bound(l2 a, l2 b, l2 c) {
	int32_t rX1 = (int32_t)((a.x + UNITS_PER_HALF_PIXEL) / UNITS_PER_PIXEL);
	int32_t rY1 = (int32_t)((a.y + UNITS_PER_HALF_PIXEL) / UNITS_PER_PIXEL);
	int32_t rX2 = (int32_t)((b.x + UNITS_PER_HALF_PIXEL) / UNITS_PER_PIXEL);
	int32_t rY2 = (int32_t)((b.y + UNITS_PER_HALF_PIXEL) / UNITS_PER_PIXEL);
	int32_t rX3 = (int32_t)((c.x + UNITS_PER_HALF_PIXEL) / UNITS_PER_PIXEL);
	int32_t rY3 = (int32_t)((c.y + UNITS_PER_HALF_PIXEL) / UNITS_PER_PIXEL);
	irect r;
	r.left = imin(imin(rX1, rX2), rX3) - 1;
	r.top = imin(imin(rY1, rY2), rY3) - 1;
	r.right = imax(imax(rX1, rX2), rX3) + 1;
	r.bottom = imax(imax(rY1, rY2), rY3) + 1;
	return r;
}

static triangle2d make_triangle(projected a, projected b, projected c) { /* ITriangle2D.cpp:51-52 */
	triangle2d t;
	t.position[0] = a; t.position[1] = b; t.position[2] = c;
	t.wholeBound = triangle_bound(a.flat, b.flat, c.flat);
	return t;
}

/* ITriangle2D::isFrontfacing (ITriangle2D.cpp:55-60). */
static int is_frontfacing(const triangle2d *t) {
	l2 a = t->position[0].flat, b = t->position[1].flat, c = t->position[2].flat;
	return ((c.x - a.x) * (b.y - a.y)) + ((c.y - a.y) * (a.x - b.x)) < 0;
}

static int rect_overlaps(irect a, irect b) { /* IRect.h:77-79 */
	return a.left < b.right && a.right > b.left && a.top < b.bottom && a.bottom > b.top;
}
static irect rect_cut(irect a, irect b) { /* IRect.h:56-66 */
	irect r = {0, 0, 0, 0};
	if (rect_overlaps(a, b)) {
		r.left = imax(a.left, b.left); r.top = imax(a.top, b.top);
		r.right = imin(a.right, b.right); r.bottom = imin(a.bottom, b.bottom);
	}
	return r;
}

/* signedModulo, roundDown, roundUp (implementation/math/scalar.h:33-49). */
static int32_t signed_modulo(int32_t a, int32_t b) { return (a >= 0) ? a % b : (b - (-a % b)) % b; }
static int32_t round_down(int32_t size, int32_t alignment) { return size - signed_modulo(size, alignment); }
static int32_t round_up(int32_t size, int32_t alignment) { return size + (alignment - 1) - signed_modulo(size - 1, alignment); }

/* getAlignedRasterBound (ITriangle2D.cpp:70-75): rows are aligned to pairs. */
static irect aligned_raster_bound(const triangle2d *t, irect clipBound) {
	irect u = rect_cut(t->wholeBound, clipBound);
	irect r = u;
	r.top = round_down(u.top, 2);
	r.bottom = round_up(u.bottom, 2);
	return r;
}

/* cutConvexEdge (ITriangle2D.cpp:86-148). */
static void cut_convex_edge(l2 s, l2 e, row_interval *rows, irect clip) {
	int32_t leftBound = clip.left, topBound = clip.top, rightBound = clip.right, bottomBound = clip.bottom;
	int64_t originX = UNITS_PER_HALF_PIXEL + (int64_t)clip.left * UNITS_PER_PIXEL;
	int64_t originY = UNITS_PER_HALF_PIXEL + (int64_t)clip.top * UNITS_PER_PIXEL;
	int64_t threshold = (s.x > e.x || (s.x == e.x && s.y > e.y)) ? -1 : 0;
	int64_t normalX = e.y - s.y;
	int64_t normalY = s.x - e.x;
	int64_t offsetX = normalX * UNITS_PER_PIXEL;
	int64_t offsetY = normalY * UNITS_PER_PIXEL;
	int64_t valueOrigin = ((originX - s.x) * normalX) + ((originY - s.y) * normalY);
	if (normalX != 0) {
		int64_t limit = threshold - valueOrigin + (offsetX * leftBound);
		if (normalX < 0) {
			for (int32_t y = topBound; y < bottomBound; y++) {
				int32_t r = y - topBound;
				int32_t leftSide = imin(imax(leftBound, (int32_t)((limit + 1) / offsetX + 1)), rightBound);
				rows[r].left = imax(rows[r].left, leftSide);
				limit -= offsetY;
			}
		} else {
			for (int32_t y = topBound; y < bottomBound; y++) {
				int32_t r = y - topBound;
				int32_t rightSide = imin(imax(leftBound, (int32_t)(limit / offsetX + 1)), rightBound);
				rows[r].right = imin(rows[r].right, rightSide);
				limit -= offsetY;
			}
		}
	} else if (normalY != 0) {
		int64_t valueRow = valueOrigin;
		for (int32_t y = topBound; y < bottomBound; y++) {
			int32_t r = y - topBound;
			if (valueRow > threshold) {
				rows[r].left = rightBound;
				rows[r].right = leftBound;
			}
			valueRow = valueRow + offsetY;
		}
	}
}

/* rasterizeTriangle (ITriangle2D.cpp:150-169). */
static void rasterize_triangle(l2 a, l2 b, l2 c, row_interval *rows, irect clip) {
	int32_t height = clip.bottom - clip.top;
	if ((a.x == b.x && a.y == b.y) || (b.x == c.x && b.y == c.y) || (c.x == a.x && c.y == a.y)) {
		for (int32_t r = 0; r < height; r++) { rows[r].left = clip.right; rows[r].right = clip.left; }
	} else {
		for (int32_t r = 0; r < height; r++) { rows[r].left = clip.left; rows[r].right = clip.right; }
		l2 p[3] = {a, b, c};
		for (int i = 0; i < 3; i++) cut_convex_edge(p[i], p[(i + 1) % 3], rows, clip);
	}
}

int32_t or_triangle_rows(const int64_t flat[6], const int32_t clip[4], int32_t *startRow, int32_t *lefts,
                         int32_t *rights, int32_t maxRows) {
	projected p[3];
	memset(p, 0, sizeof(p));
	for (int i = 0; i < 3; i++) { p[i].flat.x = flat[i * 2]; p[i].flat.y = flat[i * 2 + 1]; }
	triangle2d t = make_triangle(p[0], p[1], p[2]);
	irect clipBound = {clip[0], clip[1], clip[0] + clip[2], clip[1] + clip[3]};
	if (!rect_overlaps(t.wholeBound, clipBound)) return 0;
	irect ab = aligned_raster_bound(&t, clipBound);
	int32_t rowCount = ab.bottom - ab.top;
	if (rowCount <= 0) return 0;
	if (rowCount > maxRows) return -rowCount;
	row_interval *rows = (row_interval *)malloc(sizeof(row_interval) * rowCount);
	rasterize_triangle(p[0].flat, p[1].flat, p[2].flat, rows, ab);
	*startRow = ab.top;
	for (int32_t r = 0; r < rowCount; r++) { lefts[r] = rows[r].left; rights[r] = rows[r].right; }
	free(rows);
	return rowCount;
}

/* ------------------------------------------------------------------ projection */

typedef struct {
	int affine;
	v3 start, dx, dy; /* pWeightStart, pWeightDx, pWeightDy (ITriangle2D.h:63-78) */
} projection;

static inline float comp(v3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
static inline void setcomp(v3 *v, int i, float f) { if (i == 0) v->x = f; else if (i == 1) v->y = f; else v->z = f; }

/* ITriangle2D::getProjection (ITriangle2D.cpp:182-300). */
static projection get_projection(const triangle2d *t, v3 subB, v3 subC, int perspective) {
	v3 offsetX = {0, 0, 0}, offsetY = {0, 0, 0}, weightMultiplier = {0, 0, 0};
	v3 normalX = {0, 0, 0}, normalY = {0, 0, 0}, targetWeight = {0, 0, 0};
	for (int i = 0; i < 3; i++) {
		int j = (i + 1) % 3;
		v2 posI = t->position[i].is, posJ = t->position[j].is;
		setcomp(&offsetX, i, posJ.y - posI.y);
		setcomp(&offsetY, i, posI.x - posJ.x);
	}
	for (int i = 0; i < 3; i++) {
		int o = (i + 2) % 3;
		float otherSideValue = ((t->position[o].is.x - t->position[i].is.x) * comp(offsetX, i))
		                     + ((t->position[o].is.y - t->position[i].is.y) * comp(offsetY, i));
		setcomp(&weightMultiplier, o, (otherSideValue == 0.0f) ? 0.0f : 1.0f / otherSideValue);
	}
	for (int i = 0; i < 3; i++) {
		setcomp(&normalX, i, comp(offsetX, i) * comp(weightMultiplier, i));
		setcomp(&normalY, i, comp(offsetY, i) * comp(weightMultiplier, i));
	}
	for (int i = 0; i < 3; i++) {
		int o = (i + 2) % 3;
		setcomp(&targetWeight, o, t->position[i].is.x * -comp(normalX, i) + t->position[i].is.y * -comp(normalY, i));
	}
	v3 awdx = mk3(normalX.y, normalX.z, normalX.x);
	v3 awdy = mk3(normalY.y, normalY.z, normalY.x);
	projection p;
	if (!perspective) {
		v3 W = mk3(t->position[0].cs.z, t->position[1].cs.z, t->position[2].cs.z);
		p.affine = 1;
		p.start.x = W.x * targetWeight.x + W.y * targetWeight.y + W.z * targetWeight.z;
		p.start.y = targetWeight.x * subB.x + targetWeight.y * subB.y + targetWeight.z * subB.z;
		p.start.z = targetWeight.x * subC.x + targetWeight.y * subC.y + targetWeight.z * subC.z;
		p.dx.x = W.x * awdx.x + W.y * awdx.y + W.z * awdx.z;
		p.dx.y = awdx.x * subB.x + awdx.y * subB.y + awdx.z * subB.z;
		p.dx.z = awdx.x * subC.x + awdx.y * subC.y + awdx.z * subC.z;
		p.dy.x = W.x * awdy.x + W.y * awdy.y + W.z * awdy.z;
		p.dy.y = awdy.x * subB.x + awdy.y * subB.y + awdy.z * subB.z;
		p.dy.z = awdy.x * subC.x + awdy.y * subC.y + awdy.z * subC.z;
	} else {
		v3 IW = mk3(1.0f / t->position[0].cs.z, 1.0f / t->position[1].cs.z, 1.0f / t->position[2].cs.z);
		p.affine = 0;
		p.start.x = IW.x * targetWeight.x + IW.y * targetWeight.y + IW.z * targetWeight.z;
		p.start.y = IW.x * targetWeight.x * subB.x + IW.y * targetWeight.y * subB.y + IW.z * targetWeight.z * subB.z;
		p.start.z = IW.x * targetWeight.x * subC.x + IW.y * targetWeight.y * subC.y + IW.z * targetWeight.z * subC.z;
		p.dx.x = IW.x * awdx.x + IW.y * awdx.y + IW.z * awdx.z;
		p.dx.y = IW.x * awdx.x * subB.x + IW.y * awdx.y * subB.y + IW.z * awdx.z * subB.z;
		p.dx.z = IW.x * awdx.x * subC.x + IW.y * awdx.y * subC.y + IW.z * awdx.z * subC.z;
		p.dy.x = IW.x * awdy.x + IW.y * awdy.y + IW.z * awdy.z;
		p.dy.y = IW.x * awdy.x * subB.x + IW.y * awdy.y * subB.y + IW.z * awdy.z * subB.z;
		p.dy.z = IW.x * awdy.x * subC.x + IW.y * awdy.y * subC.y + IW.z * awdy.z * subC.z;
	}
	return p;
}

/* Projection::getWeight_affine / getDepthDividedWeight_perspective at a pixel (ITriangle2D.h:82-100). */
static v3 projection_at(const projection *p, int32_t x, int32_t y) {
	return add3(add3(p->start, scale3(p->dx, (float)x + 0.5f)), scale3(p->dy, (float)y + 0.5f));
}

/* ------------------------------------------------------------------ textures */

/* Texture constructor (implementation/image/Texture.h:66-94, 98-101). */
int or_texture_init_empty(or_texture *t, uint32_t log2w, uint32_t log2h, uint32_t maxMipLevel) {
	memset(t, 0, sizeof(*t));
	uint32_t m = maxMipLevel;
	if (log2w < m) m = log2w;
	if (log2h < m) m = log2h;
	if (m > 15u) m = 15u;
	t->log2width = log2w; t->log2height = log2h; t->maxMipLevel = m;
	uint32_t highest = (uint32_t)1 << (log2w + log2h);
	uint64_t pixelCount = 0;
	uint32_t levelPixelCount = highest;
	for (int32_t level = (int32_t)m; level >= 0; level--) {
		pixelCount = pixelCount | levelPixelCount;
		levelPixelCount = levelPixelCount >> 2;
	}
	t->startOffset = (uint32_t)pixelCount & ~highest;
	t->maxLevelMask = highest - 1;
	t->minWidthOrMask = ((uint32_t)1 << (log2w - m)) - 1;
	t->minHeightOrMask = ((uint32_t)1 << (log2h - m)) - 1;
	t->maxWidthAndMask = ((uint32_t)1 << log2w) - 1;
	t->maxHeightAndMask = ((uint32_t)1 << log2h) - 1;
	t->floatMaxWidth = (float)((uint32_t)1 << log2w);
	t->floatMaxHeight = (float)((uint32_t)1 << log2h);
	t->pixelCount = (uint32_t)pixelCount;
	t->pixels = (uint32_t *)calloc(t->pixelCount, sizeof(uint32_t));
	return t->pixels ? 0 : -1;
}

void or_texture_free(or_texture *t) {
	free(t->pixels);
	t->pixels = NULL;
}

/* texture_getPixelOffsetToLayer (api/textureAPI.h:75-85). */
uint32_t or_texture_pixel_offset_to_layer(const or_texture *t, uint32_t mipLevel) {
	return t->startOffset & (t->maxLevelMask >> (mipLevel << 1));
}

/* texture_getPixelOffset with default template arguments (textureAPI.h:102-172). */
uint32_t or_texture_pixel_offset(const or_texture *t, uint32_t x, uint32_t y, uint32_t mipLevel) {
	uint32_t tileMaskX = (t->maxWidthAndMask >> mipLevel) | t->minWidthOrMask;
	uint32_t tileMaskY = (t->maxHeightAndMask >> mipLevel) | t->minHeightOrMask;
	uint32_t log2PixelStride = t->log2width - mipLevel;
	uint32_t offset = ((y & tileMaskY) << log2PixelStride) | (x & tileMaskX);
	return or_texture_pixel_offset_to_layer(t, mipLevel) + offset;
}

uint32_t or_texture_read_pixel(const or_texture *t, uint32_t x, uint32_t y, uint32_t mipLevel) {
	return t->pixels[or_texture_pixel_offset(t, x, y, mipLevel)];
}
void or_texture_write_pixel(or_texture *t, uint32_t x, uint32_t y, uint32_t mipLevel, uint32_t color) {
	t->pixels[or_texture_pixel_offset(t, x, y, mipLevel)] = color;
}

/* downsample / texture_generatePyramid (api/textureAPI.cpp:44-63, 82-87). */
void or_texture_generate_pyramid(or_texture *t) {
	for (uint32_t level = 1; level <= t->maxMipLevel; level++) {
		uint32_t src = level - 1;
		uint32_t w = (uint32_t)1 << (t->log2width - level);
		uint32_t h = (uint32_t)1 << (t->log2height - level);
		for (uint32_t y = 0; y < h; y++) {
			for (uint32_t x = 0; x < w; x++) {
				uint32_t c[4] = {or_texture_read_pixel(t, x * 2, y * 2, src), or_texture_read_pixel(t, x * 2 + 1, y * 2, src),
				                 or_texture_read_pixel(t, x * 2, y * 2 + 1, src), or_texture_read_pixel(t, x * 2 + 1, y * 2 + 1, src)};
				uint32_t out = 0;
				for (int ch = 0; ch < 4; ch++) {
					uint32_t s = 0;
					for (int i = 0; i < 4; i++) s += (c[i] >> (ch * 8)) & 0xFFu;
					out |= (s / 4) << (ch * 8);
				}
				or_texture_write_pixel(t, x, y, level, out);
			}
		}
	}
}

/* PackOrder byte indices of red, green, blue, alpha (image/PackOrder.h:80-92). */
static const int PACK_INDEX[4][4] = {{0, 1, 2, 3}, {2, 1, 0, 3}, {1, 2, 3, 0}, {3, 2, 1, 0}};

/* ---- filter_resize(image, Sampler::Linear, width, height) (api/filterAPI.cpp:66-311, 852-859) into
 * an RGBA image, for source images in any pack order that are not sub-images, as texture creation
 * passes them.  Sampling positions are 16.16 fixed point: offset = 65536 * source / target pixels,
 * start = offset / 2 - 32768, clamped at 0, the integer part the left or upper sample.  Every path
 * reads the source's channels through its pack order (image_readPixel_clamp unpacks) and packs
 * RGBA, except the vertical-only path, whose aligned branch mixes the packed bytes as they lie
 * (mixColorsUniform), so a source of another order keeps its byte order there. */

static uint32_t resize_read(const uint32_t *img, int32_t w, int32_t h, int32_t x, int32_t y) { /* image_readPixel_clamp */
	if (x < 0) x = 0;
	if (y < 0) y = 0;
	if (x > w - 1) x = w - 1;
	if (y > h - 1) y = h - 1;
	return img[(size_t)y * w + x];
}

/* Channel ch (0 red .. 3 alpha) of a pixel packed in the given order (image_unpack). */
static uint32_t resize_channel(uint32_t c, int order, int ch) { return (c >> (PACK_INDEX[order][ch] * 8)) & 0xFFu; }

static int32_t resize_offset(int32_t source, int32_t target) { return (int32_t)((65536u * (uint32_t)source) / (uint32_t)target); }

/* Vertical only (resize_optimized, the SIMD_ALIGNED branch): mixColorsUniform with an 8-bit weight. */
static void resize_vertical(uint32_t *dst, int32_t w, int32_t h, const uint32_t *src, int32_t sh) {
	int32_t offsetY = resize_offset(sh, h);
	int32_t readY = (int32_t)((uint32_t)(offsetY / 2) - 32768u);
	for (int32_t y = 0; y < h; y++) {
		uint32_t sampleY = (uint32_t)(readY < 0 ? 0 : readY);
		uint32_t upperY = sampleY >> 16, lowerY = upperY + 1;
		if (upperY >= (uint32_t)sh) upperY = (uint32_t)sh - 1;
		if (lowerY >= (uint32_t)sh) lowerY = (uint32_t)sh - 1;
		uint32_t ratio = (sampleY & 0xFFFFu) >> 8, inv = 256u - ratio;
		for (int32_t x = 0; x < w; x++) {
			uint32_t a = src[(size_t)upperY * w + x], b = src[(size_t)lowerY * w + x], out = 0;
			for (int ch = 0; ch < 4; ch++)
				out |= ((((a >> (ch * 8)) & 0xFFu) * inv + ((b >> (ch * 8)) & 0xFFu) * ratio) >> 8) << (ch * 8);
			dst[(size_t)y * w + x] = out;
		}
		readY += offsetY;
	}
}

static uint32_t saturate_pack(const uint32_t c[4]) { /* image_saturateAndPack, RGBA */
	uint32_t out = 0;
	for (int ch = 0; ch < 4; ch++) out |= (c[ch] > 255u ? 255u : c[ch]) << (ch * 8);
	return out;
}

/* Horizontal only (resize_optimized): 16-bit weights per channel. */
static void resize_horizontal(uint32_t *dst, int32_t w, int32_t h, const uint32_t *src, int32_t sw, int order) {
	int32_t offsetX = resize_offset(sw, w);
	int32_t startX = (int32_t)((uint32_t)(offsetX / 2) - 32768u);
	for (int32_t y = 0; y < h; y++) {
		int32_t readX = startX;
		for (int32_t x = 0; x < w; x++) {
			uint32_t sampleX = (uint32_t)(readX < 0 ? 0 : readX);
			uint32_t leftX = sampleX >> 16;
			uint32_t rightRatio = sampleX & 0xFFFFu, leftRatio = 65536u - rightRatio;
			uint32_t l = resize_read(src, sw, h, (int32_t)leftX, y), r = resize_read(src, sw, h, (int32_t)(leftX + 1), y), c[4];
			for (int ch = 0; ch < 4; ch++)
				c[ch] = (resize_channel(l, order, ch) * leftRatio + resize_channel(r, order, ch) * rightRatio) >> 16;
			dst[(size_t)y * w + x] = saturate_pack(c);
			readX += offsetX;
		}
	}
}

/* Both dimensions (resize_reference with samplePixel<true>): bilinear with 16-bit weights. */
static void resize_both(uint32_t *dst, int32_t w, int32_t h, const uint32_t *src, int32_t sw, int32_t sh, int order) {
	int32_t offsetX = resize_offset(sw, w), offsetY = resize_offset(sh, h);
	int32_t startX = (int32_t)((uint32_t)(offsetX / 2) - 32768u);
	int32_t readY = (int32_t)((uint32_t)(offsetY / 2) - 32768u);
	for (int32_t y = 0; y < h; y++) {
		uint32_t sampleY = (uint32_t)(readY < 0 ? 0 : readY);
		uint32_t upperY = sampleY >> 16, lowerRatio = sampleY & 0xFFFFu, upperRatio = 65536u - lowerRatio;
		int32_t readX = startX;
		for (int32_t x = 0; x < w; x++) {
			uint32_t sampleX = (uint32_t)(readX < 0 ? 0 : readX);
			uint32_t leftX = sampleX >> 16, rightRatio = sampleX & 0xFFFFu, leftRatio = 65536u - rightRatio;
			uint32_t ul = resize_read(src, sw, sh, (int32_t)leftX, (int32_t)upperY), ur = resize_read(src, sw, sh, (int32_t)(leftX + 1), (int32_t)upperY);
			uint32_t ll = resize_read(src, sw, sh, (int32_t)leftX, (int32_t)(upperY + 1)), lr = resize_read(src, sw, sh, (int32_t)(leftX + 1), (int32_t)(upperY + 1));
			uint32_t c[4];
			for (int ch = 0; ch < 4; ch++) {
				uint32_t upper = (resize_channel(ul, order, ch) * leftRatio + resize_channel(ur, order, ch) * rightRatio) >> 16;
				uint32_t lower = (resize_channel(ll, order, ch) * leftRatio + resize_channel(lr, order, ch) * rightRatio) >> 16;
				c[ch] = (upper * upperRatio + lower * lowerRatio) >> 16;
			}
			dst[(size_t)y * w + x] = saturate_pack(c);
			readX += offsetX;
		}
		readY += offsetY;
	}
}

/* resize_optimized's choice for one step (filterAPI.cpp:157-260); the copy repacks another order
 * channel by channel (imageImpl_drawCopy, drawAPI.cpp:498-520). */
static void resize_step(uint32_t *dst, int32_t w, int32_t h, const uint32_t *src, int32_t sw, int32_t sh, int order) {
	if (sw == w && sh == h) {
		if (order == 0) {
			memcpy(dst, src, sizeof(uint32_t) * (size_t)w * (size_t)h);
		} else {
			for (size_t i = 0; i < (size_t)w * (size_t)h; i++) {
				uint32_t out = 0;
				for (int ch = 0; ch < 4; ch++) out |= resize_channel(src[i], order, ch) << (ch * 8);
				dst[i] = out;
			}
		}
	}
	else if (sw == w) resize_vertical(dst, w, h, src, sh);
	else if (sh == h) resize_horizontal(dst, w, h, src, sw, order);
	else resize_both(dst, w, h, src, sw, sh, order);
}

/* resizeToTarget (filterAPI.cpp:298-314): a wider and taller target goes through a horizontal step
 * to the target's width first, into an RGBA image. */
void or_filter_resize_linear_ordered(uint32_t *dst, int32_t w, int32_t h, const uint32_t *src, int32_t sw, int32_t sh, int32_t srcOrder) {
	if (w != sw && h > sh) {
		uint32_t *temp = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)w * (size_t)sh);
		resize_step(temp, w, sh, src, sw, sh, srcOrder);
		resize_step(dst, w, h, temp, w, sh, 0);
		free(temp);
	} else {
		resize_step(dst, w, h, src, sw, sh, srcOrder);
	}
}

void or_filter_resize_linear(uint32_t *dst, int32_t w, int32_t h, const uint32_t *src, int32_t sw, int32_t sh) {
	or_filter_resize_linear_ordered(dst, w, h, src, sw, sh, 0);
}

/* findLog2Size (textureAPI.cpp:30-40). */
static uint32_t find_log2_size(uint32_t size) {
	for (uint32_t l = 0; l < 15u; l++) if (((uint32_t)1 << l) >= size) return l;
	return 15u;
}

/* texture_create_RgbaU8(image, resolutions) (textureAPI.cpp:89-110, 112-131): the image resized
 * linearly to the next powers of two, then the pyramid. */
int or_texture_create_from_image_ordered(or_texture *t, const uint32_t *level0, int32_t width, int32_t height, int32_t resolutions,
                                         int32_t packOrder) {
	if (resolutions < 1 || width < 1 || height < 1 || width > 32768 || height > 32768 || packOrder < 0 || packOrder > 3) return -1;
	uint32_t lw = find_log2_size((uint32_t)width), lh = find_log2_size((uint32_t)height);
	if (or_texture_init_empty(t, lw, lh, (uint32_t)(resolutions - 1))) return -1;
	uint32_t base = or_texture_pixel_offset_to_layer(t, 0);
	or_filter_resize_linear_ordered(t->pixels + base, (int32_t)1 << lw, (int32_t)1 << lh, level0, width, height, packOrder);
	or_texture_generate_pyramid(t);
	return 0;
}

int or_texture_create_from_image(or_texture *t, const uint32_t *level0, int32_t width, int32_t height, int32_t resolutions) {
	return or_texture_create_from_image_ordered(t, level0, width, height, resolutions, 0);
}

/* weightColors (textureAPI.h:242-255): per channel (a*wa + b*wb) >> 8. */
static uint32_t weight_colors(uint32_t a, uint32_t wa, uint32_t b, uint32_t wb) {
	uint32_t out = 0;
	for (int ch = 0; ch < 4; ch++) {
		uint32_t ca = (a >> (ch * 8)) & 0xFFu, cb = (b >> (ch * 8)) & 0xFFu;
		uint32_t mixed = ((ca * wa + cb * wb) & 0xFFFFu) >> 8;
		out |= (mixed & 0xFFu) << (ch * 8);
	}
	return out;
}

/* texture_interpolate_color_linear (textureAPI.h:284-292). */
uint32_t or_interpolate_color_linear(uint32_t a, uint32_t b, uint32_t weight) {
	return weight_colors(a, 256u - weight, b, weight);
}

/* texture_interpolate_color_bilinear (textureAPI.h:310-318). */
uint32_t or_interpolate_color_bilinear(uint32_t a, uint32_t b, uint32_t c, uint32_t d, uint32_t wx, uint32_t wy) {
	return weight_colors(weight_colors(a, 256u - wx, b, wx), 256u - wy, weight_colors(c, 256u - wx, d, wx), wy);
}

/* texture_sample_bilinear with MIP_INSIDE (textureAPI.h:320-430). */
uint32_t or_sample_bilinear(const or_texture *t, float u, float v, uint32_t mipLevel, int highestResolution) {
	uint32_t scaleU = 256u << t->log2width;
	uint32_t scaleV = 256u << t->log2height;
	uint32_t maskX = t->maxWidthAndMask, maskY = t->maxHeightAndMask;
	uint32_t log2Stride = t->log2width;
	uint32_t layer = t->startOffset;
	if (!highestResolution) {
		scaleU >>= mipLevel; scaleV >>= mipLevel;
		maskX >>= mipLevel; maskY >>= mipLevel;
		log2Stride -= mipLevel;
		layer = or_texture_pixel_offset_to_layer(t, mipLevel);
	}
	uint32_t subCenterX = trunc_u32((u + 256.0f) * (float)scaleU) - 128u;
	uint32_t subCenterY = trunc_u32((v + 256.0f) * (float)scaleV) - 128u;
	uint32_t weightX = subCenterX & 0xFFu, weightY = subCenterY & 0xFFu;
	uint32_t left = subCenterX >> 8, top = subCenterY >> 8;
	uint32_t right = (left + 1u) & maskX, bottom = (top + 1u) & maskY;
	left &= maskX; top &= maskY;
	uint32_t upper = top << log2Stride, lower = bottom << log2Stride;
	uint32_t a = t->pixels[(upper | left) + layer];
	uint32_t b = t->pixels[(upper | right) + layer];
	uint32_t c = t->pixels[(lower | left) + layer];
	uint32_t d = t->pixels[(lower | right) + layer];
	return or_interpolate_color_bilinear(a, b, c, d, weightX, weightY);
}

/* texture_sample_nearest with its default template arguments (api/textureAPI.h:218-236): the mip level
 * is not assumed inside the pyramid, so texel coordinates are tiled with the clamped masks of
 * texture_getPixelOffset. */
uint32_t or_sample_nearest(const or_texture *t, float u, float v, uint32_t mipLevel, int highestResolution) {
	uint32_t scaleU = 1u << t->log2width, scaleV = 1u << t->log2height;
	if (!highestResolution) { scaleU >>= mipLevel; scaleV >>= mipLevel; }
	uint32_t x = trunc_u32((u + 256.0f) * (float)scaleU);
	uint32_t y = trunc_u32((v + 256.0f) * (float)scaleV);
	return or_texture_read_pixel(t, x, y, highestResolution ? 0u : mipLevel);
}

/* texture_getMipLevelIndex (textureAPI.h:471-495) on lanes 0 (upper left), 1 (upper right), 2 (lower left). */
uint32_t or_mip_level_index(const or_texture *t, const float u[4], const float v[4]) {
	float offsetUX = fabsf(u[0] - u[1]);
	float offsetUY = fabsf(u[0] - u[2]);
	float offsetVX = fabsf(v[0] - v[1]);
	float offsetVY = fabsf(v[0] - v[2]);
	float offsetU = fmaxf_ref(offsetUX, offsetUY) * t->floatMaxWidth;
	float offsetV = fmaxf_ref(offsetVX, offsetVY) * t->floatMaxHeight;
	float offset = fmaxf_ref(offsetU, offsetV);
	int32_t result = 0;
	if (offset > 2.0f) result = 1;
	if (offset > 4.0f) result = 2;
	if (offset > 8.0f) result = 3;
	if (offset > 16.0f) result = 4;
	if (result > (int32_t)t->maxMipLevel) result = (int32_t)t->maxMipLevel;
	return (uint32_t)result;
}

/* ------------------------------------------------------------------ shading */

typedef struct {
	const or_texture *diffuse, *light;
	v3 u1, v1, u2, v2;            /* TriangleTexCoords (shader/Shader.h:36-45) */
	v3 red, green, blue, alpha;   /* scaled TriangleColors (Shader.h:47-60) */
	int hasDiffuse, diffuseSingleLayer, hasLight, hasVertexFade, colorless;
} shade_data;

static int almost_zero(float v) { return v > -0.001f && v < 0.001f; }               /* fillerTemplates.h:37-39 */
static int almost_one(float v) { return v > 0.999f && v < 1.001f; }                 /* fillerTemplates.h:45-47 */
static int almost_zero3(v3 c) { return almost_zero(c.x) && almost_zero(c.y) && almost_zero(c.z); }
static int almost_one3(v3 c) { return almost_one(c.x) && almost_one(c.y) && almost_one(c.z); }
static int almost_same3(v3 c) { return almost_zero(c.x - c.y) && almost_zero(c.x - c.z) && almost_zero(c.y - c.z); }

/* RgbaMultiply_data + processTriangle_RgbaMultiply's variant selection (shader/RgbaMultiply.h:37-58, 110-173). */
static void shade_setup(shade_data *d, const or_texture *diffuse, const or_texture *light,
                        const float *tc0, const float *tc1, const float *tc2,
                        const float *c0, const float *c1, const float *c2) {
	d->diffuse = diffuse; d->light = light;
	d->u1 = mk3(tc0[0], tc1[0], tc2[0]); d->v1 = mk3(tc0[1], tc1[1], tc2[1]);
	d->u2 = mk3(tc0[2], tc1[2], tc2[2]); d->v2 = mk3(tc0[3], tc1[3], tc2[3]);
	float scale = 255.0f;
	if (diffuse) scale *= 1.0f / 255.0f;
	if (light) scale *= 1.0f / 255.0f;
	d->red = scale3(mk3(c0[0], c1[0], c2[0]), scale);
	d->green = scale3(mk3(c0[1], c1[1], c2[1]), scale);
	d->blue = scale3(mk3(c0[2], c1[2], c2[2]), scale);
	d->alpha = scale3(mk3(c0[3], c1[3], c2[3]), scale);
	d->hasVertexFade = !(almost_same3(d->red) && almost_same3(d->green) && almost_same3(d->blue) && almost_same3(d->alpha));
	d->colorless = almost_one3(d->red) && almost_one3(d->green) && almost_one3(d->blue) && almost_one3(d->alpha);
	d->hasDiffuse = diffuse != NULL;
	d->diffuseSingleLayer = diffuse ? (diffuse->maxMipLevel == 0) : 0;
	d->hasLight = light != NULL;
	/* With both textures, colorless is not a separate variant (RgbaMultiply.h:118-133). */
	if (d->hasDiffuse && d->hasLight) d->colorless = 0;
	/* Without textures, a colorless-looking triangle still takes the constant-colour variant. */
	if (!d->hasDiffuse && !d->hasLight) d->colorless = 0;
	if (d->hasVertexFade) d->colorless = 0;
}

/* shaderMethods::interpolate (shader/shaderMethods.h:39-45). */
static inline float interpolate(v3 data, float wa, float wb, float wc) {
	float a = data.x * wa, b = data.y * wb, c = data.z * wc;
	return a + b + c;
}

static void unpack_rgba(uint32_t c, float out[4]) { /* Rgba_F32(U32x4) (shader/shaderTypes.h:40-45) */
	out[0] = (float)(c & 0xFFu); out[1] = (float)((c >> 8) & 0xFFu);
	out[2] = (float)((c >> 16) & 0xFFu); out[3] = (float)(c >> 24);
}

static void sample_quad(const or_texture *t, const float u[4], const float v[4], int highest, float rgba[4][4]) {
	uint32_t mip = highest ? 0u : or_mip_level_index(t, u, v);
	for (int l = 0; l < 4; l++) unpack_rgba(or_sample_bilinear(t, u[l], v[l], mip, highest), rgba[l]);
}

/* getPixels_2x2 (shader/RgbaMultiply.h:74-106): out[lane][channel]. */
static void shade_quad(const shade_data *d, const float wa[4], const float wb[4], const float wc[4], float out[4][4]) {
	float u[4], v[4];
	if (d->hasDiffuse && !d->hasLight && d->colorless) {
		for (int l = 0; l < 4; l++) { u[l] = interpolate(d->u1, wa[l], wb[l], wc[l]); v[l] = interpolate(d->v1, wa[l], wb[l], wc[l]); }
		sample_quad(d->diffuse, u, v, 0, out);
		return;
	}
	if (d->hasLight && !d->hasDiffuse && d->colorless) {
		for (int l = 0; l < 4; l++) { u[l] = interpolate(d->u2, wa[l], wb[l], wc[l]); v[l] = interpolate(d->v2, wa[l], wb[l], wc[l]); }
		sample_quad(d->light, u, v, 1, out);
		return;
	}
	for (int l = 0; l < 4; l++) {
		if (d->hasVertexFade) {
			out[l][0] = interpolate(d->red, wa[l], wb[l], wc[l]);
			out[l][1] = interpolate(d->green, wa[l], wb[l], wc[l]);
			out[l][2] = interpolate(d->blue, wa[l], wb[l], wc[l]);
			out[l][3] = interpolate(d->alpha, wa[l], wb[l], wc[l]);
		} else {
			out[l][0] = d->red.x; out[l][1] = d->green.x; out[l][2] = d->blue.x; out[l][3] = d->alpha.x;
		}
	}
	float s[4][4];
	if (d->hasDiffuse) {
		for (int l = 0; l < 4; l++) { u[l] = interpolate(d->u1, wa[l], wb[l], wc[l]); v[l] = interpolate(d->v1, wa[l], wb[l], wc[l]); }
		sample_quad(d->diffuse, u, v, 0, s);
		for (int l = 0; l < 4; l++) for (int ch = 0; ch < 4; ch++) out[l][ch] = out[l][ch] * s[l][ch];
	}
	if (d->hasLight) {
		for (int l = 0; l < 4; l++) { u[l] = interpolate(d->u2, wa[l], wb[l], wc[l]); v[l] = interpolate(d->v2, wa[l], wb[l], wc[l]); }
		sample_quad(d->light, u, v, 1, s);
		for (int l = 0; l < 4; l++) for (int ch = 0; ch < 4; ch++) out[l][ch] = out[l][ch] * s[l][ch];
	}
}

/* packOrder_floatToSaturatedByte with an order (PackOrder.h:204-212). */
static uint32_t pack_saturated(const float rgba[4], int packOrder) {
	uint32_t out = 0;
	for (int ch = 0; ch < 4; ch++) {
		float c = rgba[ch];
		float clamped = (255.1f < c) ? 255.1f : c; /* clampUpper via min (noSimd.h:183-185, simd.h:2198-2215) */
		out |= trunc_u32(clamped) << (PACK_INDEX[packOrder][ch] * 8);
	}
	return out;
}

static void unpack_ordered(uint32_t c, int packOrder, float out[4]) { /* Rgba_F32(U, order) (shaderTypes.h:46-50) */
	for (int ch = 0; ch < 4; ch++) out[ch] = (float)((c >> (PACK_INDEX[packOrder][ch] * 8)) & 0xFFu);
}

/* ------------------------------------------------------------------ filler */

typedef struct {
	uint32_t *color; float *depth;
	int32_t width, height;
	int packOrder;
	or_stats *stats;
	uint32_t key;
	uint64_t fragments;
} target;

/* fillQuadSuper (shader/fillerTemplates.h:154-187) for one 2x2 quad at x. */
static void fill_quad(target *tg, const shade_data *sd, int clipSides, int colorWrite, int depthRead, int depthWrite,
                      int alphaFilter, int affine, int32_t x, int32_t yUpper, int32_t yLower, row_interval upper, row_interval lower,
                      const float depth[4], const float wa[4], const float wb[4], const float wc[4]) {
	/* Lanes of a missing lower row (the last row pair of an odd height) point at the upper row: a
	 * full quad tests and writes them there, but they add no (pixel, triangle) pair of their own to
	 * the fragment statistics, whose upper lane already holds that pair. */
	const int lowerAliased = (yLower == yUpper) && clipSides == 0;
	int clip[4];
	if (clipSides) {
		int32_t x2 = x + 1;
		clip[0] = x >= upper.left && x < upper.right;
		clip[1] = x2 >= upper.left && x2 < upper.right;
		clip[2] = x >= lower.left && x < lower.right;
		clip[3] = x2 >= lower.left && x2 < lower.right;
	} else {
		clip[0] = clip[1] = clip[2] = clip[3] = 1;
	}
	size_t idx[4] = {(size_t)yUpper * tg->width + x, (size_t)yUpper * tg->width + x + 1,
	                 (size_t)yLower * tg->width + x, (size_t)yLower * tg->width + x + 1};
	int vis[4];
	for (int l = 0; l < 4; l++) {
		int front = 1;
		if (depthRead) {
			if (clipSides && !clip[l]) {
				front = 0;
			} else {
				float old = tg->depth[idx[l]];
				front = affine ? (depth[l] < old) : (depth[l] > old);
			}
		}
		vis[l] = clip[l] && front;
		if (clip[l] && !(lowerAliased && l >= 2)) {
			tg->fragments++;
			if (tg->stats && tg->stats->coverage) tg->stats->coverage[idx[l]]++;
		}
	}
	if (!(vis[0] || vis[1] || vis[2] || vis[3])) return;
	if (colorWrite) {
		float src[4][4];
		shade_quad(sd, wa, wb, wc, src);
		if (alphaFilter) {
			for (int l = 0; l < 4; l++) {
				float opacity = src[l][3] * (1.0f / 255.0f);
				float dst[4];
				uint32_t packed = (clipSides && !vis[l]) ? 0u : tg->color[idx[l]];
				unpack_ordered(packed, tg->packOrder, dst);
				for (int ch = 0; ch < 4; ch++) src[l][ch] = (src[l][ch] * opacity) + (dst[ch] * (1.0f - opacity));
			}
		}
		for (int l = 0; l < 4; l++) {
			uint32_t packed = pack_saturated(src[l], tg->packOrder);
			if (vis[l]) {
				tg->color[idx[l]] = packed;
				if (tg->stats && tg->stats->winner) tg->stats->winner[idx[l]] = tg->key;
			}
		}
	}
	if (depthWrite) {
		for (int l = 0; l < 4; l++) {
			if (vis[l]) {
				tg->depth[idx[l]] = depth[l];
				if (!colorWrite && tg->stats && tg->stats->winner) tg->stats->winner[idx[l]] = tg->key;
			}
		}
	}
}

/* fillRowSuper (fillerTemplates.h:195-244) over quads [startX, endX). */
static void fill_row(target *tg, const shade_data *sd, int clipSides, int colorWrite, int depthRead, int depthWrite,
                     int alphaFilter, int affine, v3 pUpper, v3 pLower, v3 pDx, int32_t startX, int32_t endX,
                     int32_t yUpper, int32_t yLower, row_interval upper, row_interval lower) {
	v3 dx2 = scale3(pDx, 2.0f);
	float a[4] = {pUpper.x, pUpper.x + pDx.x, pLower.x, pLower.x + pDx.x};
	float b[4] = {pUpper.y, pUpper.y + pDx.y, pLower.y, pLower.y + pDx.y};
	float c[4] = {pUpper.z, pUpper.z + pDx.z, pLower.z, pLower.z + pDx.z};
	for (int32_t x = startX; x < endX; x += 2) {
		float depth[4], wa[4], wb[4], wc[4];
		for (int l = 0; l < 4; l++) {
			depth[l] = a[l];
			if (affine) {
				wb[l] = b[l];
				wc[l] = c[l];
			} else {
				float linearDepth = 1.0f / a[l]; /* reciprocal, scalar build (noSimd.h:187, simd.h:4063-4066) */
				wb[l] = b[l] * linearDepth;
				wc[l] = c[l] * linearDepth;
			}
			wa[l] = 1.0f - (wb[l] + wc[l]);
		}
		fill_quad(tg, sd, clipSides, colorWrite, depthRead, depthWrite, alphaFilter, affine, x, yUpper, yLower, upper, lower, depth, wa, wb, wc);
		for (int l = 0; l < 4; l++) { a[l] = a[l] + dx2.x; b[l] = b[l] + dx2.y; c[l] = c[l] + dx2.z; }
	}
}

static inline int32_t round_up_even(int32_t x) { return (int32_t)(((uint32_t)x + 1u) & ~1u); } /* fillerTemplates.h:57-59 */
static inline int32_t round_down_even(int32_t x) { return (int32_t)((uint32_t)x & ~1u); }      /* fillerTemplates.h:61-63 */

/* fillShapeSuper (fillerTemplates.h:246-385). */
static void fill_shape(target *tg, const shade_data *sd, const projection *proj, int32_t startRow, int32_t rowCount,
                       const row_interval *rows, int colorWrite, int depthRead, int depthWrite, int alphaFilter) {
	int affine = proj->affine;
	v3 doubleDx = scale3(proj->dx, 2.0f);
	int32_t maxHeight = tg->height;
	for (int32_t y1 = startRow; y1 < startRow + rowCount; y1 += 2) {
		int32_t y2 = y1 + 1;
		row_interval upper = rows[y1 - startRow];
		row_interval lower = rows[y2 - startRow];
		int32_t outerStart = imin(upper.left, lower.left);
		int32_t outerEnd = imax(upper.right, lower.right);
		int32_t innerStart = imax(upper.left, lower.left);
		int32_t innerEnd = imin(upper.right, lower.right);
		int32_t obs = round_down_even(outerStart), obe = round_up_even(outerEnd);
		int32_t ibs = round_up_even(innerStart), ibe = round_down_even(innerEnd);
		if (y2 >= maxHeight) lower.right = lower.left;
		int hasTop = upper.right > upper.left;
		int hasBottom = lower.right > lower.left;
		if (!(hasTop || hasBottom)) continue;
		/* Rows that are missing read and write the other row of the pair (fillerTemplates.h:295-327). */
		int32_t yUpper = hasTop ? y1 : y2;
		int32_t yLower = hasBottom ? y2 : y1;
		v3 pUpper = projection_at(proj, obs, y1);
		v3 pLower = add3(pUpper, proj->dy);
		if (ibe <= ibs) {
			for (int32_t x = obs; x < obe; x += 2) {
				fill_row(tg, sd, 1, colorWrite, depthRead, depthWrite, alphaFilter, affine, pUpper, pLower, proj->dx, x, x + 2, yUpper, yLower, upper, lower);
				pUpper = add3(pUpper, doubleDx); pLower = add3(pLower, doubleDx);
			}
		} else {
			for (int32_t x = obs; x < ibs; x += 2) {
				fill_row(tg, sd, 1, colorWrite, depthRead, depthWrite, alphaFilter, affine, pUpper, pLower, proj->dx, x, x + 2, yUpper, yLower, upper, lower);
				pUpper = add3(pUpper, doubleDx); pLower = add3(pLower, doubleDx);
			}
			int32_t quadCount = (ibe - ibs) / 2;
			row_interval none = {0, 0};
			fill_row(tg, sd, 0, colorWrite, depthRead, depthWrite, alphaFilter, affine, pUpper, pLower, proj->dx, ibs, ibe, yUpper, yLower, none, none);
			pUpper = add3(pUpper, scale3(doubleDx, (float)quadCount));
			pLower = add3(pLower, scale3(doubleDx, (float)quadCount));
			for (int32_t x = ibe; x < obe; x += 2) {
				fill_row(tg, sd, 1, colorWrite, depthRead, depthWrite, alphaFilter, affine, pUpper, pLower, proj->dx, x, x + 2, yUpper, yLower, upper, lower);
				pUpper = add3(pUpper, doubleDx); pLower = add3(pLower, doubleDx);
			}
		}
	}
}

/* ------------------------------------------------------------------ draw commands */

typedef struct {
	triangle2d triangle;
	v3 subB, subC;
	shade_data shade;
	int filter;
	uint32_t key; /* submission order: triangle index * 8 + clipped sub-triangle index */
	int32_t task; /* renderer task (camera) of the command */
	int occluded; /* TriangleDrawCommand::occluded (renderCore.h:67) */
} command;

typedef struct {
	command *items;
	size_t count, capacity;
} command_list;

static void push_command(command_list *list, const command *c) {
	if (list->count == list->capacity) {
		size_t cap = list->capacity ? list->capacity * 2 : 1024;
		list->items = (command *)realloc(list->items, cap * sizeof(command));
		list->capacity = cap;
	}
	list->items[list->count++] = *c;
}

/* getTriangleVisibility (renderCore.cpp:172-198): 0 Hidden, 1 Full, 2 Partial. */
static int triangle_visibility(const triangle2d *t, const camera *c, int clipFrustum) {
	int planeCount = clipFrustum ? c->clipCount : c->cullCount;
	const plane3 *planes = clipFrustum ? c->clip : c->cull;
	int outside[3][6];
	for (int k = 0; k < 3; k++)
		for (int s = 0; s < planeCount; s++) outside[k][s] = !plane_inside(&planes[s], t->position[k].cs);
	for (int s = 0; s < planeCount; s++)
		if (outside[0][s] && outside[1][s] && outside[2][s]) return 0;
	for (int k = 0; k < 3; k++)
		for (int s = 0; s < planeCount; s++)
			if (outside[k][s]) return 2;
	return 1;
}

typedef struct { v3 cs; float subB, subC; int state; float value; } sub_vertex; /* renderCore.cpp:33-47 */

static sub_vertex sub_lerp(sub_vertex a, sub_vertex b, float ratio) {
	sub_vertex r;
	float inv = 1.0f - ratio;
	r.cs = add3(scale3(a.cs, inv), scale3(b.cs, ratio));
	r.subB = a.subB * inv + b.subB * ratio;
	r.subC = a.subC * inv + b.subC * ratio;
	r.state = 0; r.value = 0.0f;
	return r;
}

static float inverse_lerp(float a, float b, float value) { /* renderCore.cpp:52-59 */
	float c = b - a;
	return (c == 0.0f) ? 0.5f : (value - a) / c;
}

#define MAX_POINTS 9
typedef struct { int count; sub_vertex v[MAX_POINTS]; } clipped_triangle;

static void clipped_delete(clipped_triangle *ct, int index) { /* renderCore.cpp:76-86 */
	if (ct->count > 0 && ct->count <= MAX_POINTS) {
		for (int v = index; v < ct->count - 1; v++) ct->v[v] = ct->v[v + 1];
		ct->count--;
	}
}
static void clipped_insert(clipped_triangle *ct, int index, sub_vertex nv) { /* renderCore.cpp:87-99 */
	if (ct->count < MAX_POINTS) {
		for (int v = ct->count - 1; v >= index; v--) ct->v[v + 1] = ct->v[v];
		ct->v[index] = nv;
		ct->count++;
	}
}

/* ClippedTriangle::clip (renderCore.cpp:104-169). */
static void clipped_clip(clipped_triangle *ct, const plane3 *p) {
	if (!(ct->count >= 3 && ct->count < MAX_POINTS)) return;
	int outsideCount = 0, lastOutside = 0;
	for (int v = 0; v < ct->count; v++) {
		float distance = dot3(p->normal, ct->v[v].cs) - p->offset;
		ct->v[v].value = distance;
		if (distance > 0.0f) { outsideCount++; lastOutside = v; ct->v[v].state = 1; } else { ct->v[v].state = 0; }
	}
	if (outsideCount == 0) return;
	if (outsideCount >= ct->count) {
		ct->count = 0;
	} else if (outsideCount == 1) {
		int cur = lastOutside;
		int prev = (lastOutside - 1 + ct->count) % ct->count;
		int next = (lastOutside + 1) % ct->count;
		float r0 = inverse_lerp(ct->v[prev].value, ct->v[cur].value, 0.0f);
		float r1 = inverse_lerp(ct->v[cur].value, ct->v[next].value, 0.0f);
		sub_vertex cutStart = sub_lerp(ct->v[prev], ct->v[cur], r0);
		sub_vertex cutEnd = sub_lerp(ct->v[cur], ct->v[next], r1);
		ct->v[lastOutside] = cutStart;
		clipped_insert(ct, next, cutEnd);
	} else {
		for (int cur = 0; cur < ct->count; cur++) {
			int prev = (cur - 1 + ct->count) % ct->count;
			int next = (cur + 1) % ct->count;
			if (ct->v[cur].state == 1) {
				if (ct->v[prev].state == 0) {
					float r = inverse_lerp(ct->v[prev].value, ct->v[cur].value, 0.0f);
					ct->v[cur] = sub_lerp(ct->v[prev], ct->v[cur], r);
					ct->v[cur].state = 2;
				} else if (ct->v[next].state == 0) {
					float r = inverse_lerp(ct->v[cur].value, ct->v[next].value, 0.0f);
					ct->v[cur] = sub_lerp(ct->v[cur], ct->v[next], r);
					ct->v[cur].state = 2;
				}
			}
		}
		if (outsideCount > 2) {
			for (int v = ct->count - 1; v >= 0; v--)
				if (ct->v[v].state == 1) clipped_delete(ct, v);
		}
	}
}

/* renderTriangleFromData + renderTriangleWithShader + drawClippedTriangle + drawSubTriangle
 * (renderCore.cpp:220-341): emits draw commands for one triangle. */
static void submit_triangle(command_list *out, const camera *cam, int hasColor, int hasDepth, int32_t width, int32_t height,
                            projected a, projected b, projected c, int filter, const or_texture *diffuse, const or_texture *light,
                            const float *tc0, const float *tc1, const float *tc2, const float *c0, const float *c1, const float *c2,
                            uint32_t triangleIndex) {
	(void)width; (void)height;
	if (!hasColor && !hasDepth) return;
	triangle2d tri = make_triangle(a, b, c);
	if (triangle_visibility(&tri, cam, 0) == 0) return;
	if (filter == 1 && almost_zero3(mk3(c0[3], c1[3], c2[3]))) return;
	command cmd;
	memset(&cmd, 0, sizeof(cmd));
	shade_setup(&cmd.shade, diffuse, light, tc0, tc1, tc2, c0, c1, c2);
	cmd.filter = filter;
	if (triangle_visibility(&tri, cam, 1) == 1) {
		if (is_frontfacing(&tri)) {
			cmd.triangle = tri;
			cmd.subB = mk3(0.0f, 1.0f, 0.0f);
			cmd.subC = mk3(0.0f, 0.0f, 1.0f);
			cmd.key = triangleIndex * 8u;
			push_command(out, &cmd);
		}
	} else {
		clipped_triangle ct;
		memset(&ct, 0, sizeof(ct));
		ct.v[0].cs = tri.position[0].cs; ct.v[0].subB = 0.0f; ct.v[0].subC = 0.0f;
		ct.v[1].cs = tri.position[1].cs; ct.v[1].subB = 1.0f; ct.v[1].subC = 0.0f;
		ct.v[2].cs = tri.position[2].cs; ct.v[2].subB = 0.0f; ct.v[2].subC = 1.0f;
		ct.count = 3;
		for (int s = 0; s < cam->clipCount; s++) clipped_clip(&ct, &cam->clip[s]);
		for (int k = 0; k < ct.count - 2; k++) {
			sub_vertex va = ct.v[0], vb = ct.v[1 + k], vc = ct.v[2 + k];
			triangle2d sub = make_triangle(camera_to_screen(cam, va.cs), camera_to_screen(cam, vb.cs), camera_to_screen(cam, vc.cs));
			if (is_frontfacing(&sub)) {
				cmd.triangle = sub;
				cmd.subB = mk3(va.subB, vb.subB, vc.subB);
				cmd.subC = mk3(va.subC, vb.subC, vc.subC);
				cmd.key = triangleIndex * 8u + (uint32_t)k;
				push_command(out, &cmd);
			}
		}
	}
}

/* executeTriangleDrawing (renderCore.cpp:203-217) then processTriangle_RgbaMultiply + fillShape
 * (RgbaMultiply.h:110-175, fillerTemplates.h:387-441). */
static void execute_command(const command *cmd, const camera *cam, target *tg, irect imageBound, irect band,
                            row_interval **rowBuffer, int32_t *rowCapacity) {
	irect finalClip = rect_cut(imageBound, band);
	if (!rect_overlaps(cmd->triangle.wholeBound, finalClip)) return;
	irect ab = aligned_raster_bound(&cmd->triangle, finalClip);
	int32_t rowCount = ab.bottom - ab.top;
	if (rowCount <= 0) return;
	if (rowCount > *rowCapacity) {
		*rowBuffer = (row_interval *)realloc(*rowBuffer, sizeof(row_interval) * rowCount);
		*rowCapacity = rowCount;
	}
	rasterize_triangle(cmd->triangle.position[0].flat, cmd->triangle.position[1].flat, cmd->triangle.position[2].flat, *rowBuffer, ab);
	projection proj = get_projection(&cmd->triangle, cmd->subB, cmd->subC, cam->perspective);
	int hasColor = tg->color != NULL, hasDepth = tg->depth != NULL;
	/* fillShape's choice of fillShapeSuper instance (fillerTemplates.h:387-441). */
	int colorWrite = hasColor;
	int depthRead = hasDepth;
	int depthWrite = hasDepth && !(hasColor && cmd->filter != 0);
	int alphaFilter = hasColor && cmd->filter != 0;
	if (!hasColor && !hasDepth) return;
	tg->key = cmd->key;
	fill_shape(tg, &cmd->shade, &proj, ab.top, rowCount, *rowBuffer, colorWrite, depthRead, depthWrite, alphaFilter);
	if (tg->stats) tg->stats->trianglesDrawn++;
}

typedef struct {
	const command_list *commands;
	const camera *cam;
	target base;
	irect imageBound;
	irect *bands;
	int32_t bandCount;
	int32_t nextBand;
	pthread_mutex_t lock;
	uint64_t fragments;
	uint64_t drawn;
} band_job;

static void *band_worker(void *arg) {
	band_job *job = (band_job *)arg;
	row_interval *rows = NULL;
	int32_t capacity = 0;
	or_stats localStats;
	for (;;) {
		pthread_mutex_lock(&job->lock);
		int32_t b = job->nextBand++;
		pthread_mutex_unlock(&job->lock);
		if (b >= job->bandCount) break;
		target tg = job->base;
		memset(&localStats, 0, sizeof(localStats));
		if (job->base.stats) {
			localStats.coverage = job->base.stats->coverage;
			localStats.winner = job->base.stats->winner;
		}
		tg.stats = &localStats;
		tg.fragments = 0;
		for (size_t i = 0; i < job->commands->count; i++)
			execute_command(&job->commands->items[i], job->cam, &tg, job->imageBound, job->bands[b], &rows, &capacity);
		pthread_mutex_lock(&job->lock);
		job->fragments += tg.fragments;
		job->drawn += localStats.trianglesDrawn;
		pthread_mutex_unlock(&job->lock);
	}
	free(rows);
	return NULL;
}

static void model_bound(const or_model *m, v3 *mn, v3 *mx) { /* ModelImpl::expandBound from a zero bound (Model.cpp:281-288) */
	*mn = mk3(0.0f, 0.0f, 0.0f); *mx = mk3(0.0f, 0.0f, 0.0f);
	for (int32_t i = 0; i < m->pointCount; i++) {
		const float *p = m->positions + i * 3;
		if (mn->x > p[0]) mn->x = p[0];
		if (mn->y > p[1]) mn->y = p[1];
		if (mn->z > p[2]) mn->z = p[2];
		if (mx->x < p[0]) mx->x = p[0];
		if (mx->y < p[1]) mx->y = p[1];
		if (mx->z < p[2]) mx->z = p[2];
	}
}

int or_model_render(const or_model *model, const float modelToWorld[12], const or_camera_desc *desc,
                    uint32_t *color, float *depth, int32_t packOrder, int32_t bands, int32_t threads, or_stats *stats) {
	camera cam;
	camera_create(&cam, desc);
	v3 mn, mx;
	model_bound(model, &mn, &mx);
	if (!box_seen(&cam, mn, mx, modelToWorld)) return 0; /* ModelImpl::render (Model.cpp:185-197) */
	projected *proj = (projected *)malloc(sizeof(projected) * (size_t)(model->pointCount > 0 ? model->pointCount : 1));
	for (int32_t i = 0; i < model->pointCount; i++) {
		v3 p = mk3(model->positions[i * 3], model->positions[i * 3 + 1], model->positions[i * 3 + 2]);
		proj[i] = camera_to_screen(&cam, world_to_camera(&cam, transform_point(modelToWorld, p)));
	}
	command_list commands = {NULL, 0, 0};
	uint32_t triangleIndex = 0;
	for (int32_t p = 0; p < model->polyCount; p++) { /* Part::render (Model.cpp:150-162), fan (Model.cpp:135-148) */
		const int32_t *idx = model->polyIndices + p * 4;
		int triCount = (idx[3] < 0) ? 1 : 2;
		for (int t = 0; t < triCount; t++) {
			int ia = 0, ib = 1 + t, ic = 2 + t;
			submit_triangle(&commands, &cam, color != NULL, depth != NULL, desc->width, desc->height,
			                proj[idx[ia]], proj[idx[ib]], proj[idx[ic]], model->filter, model->diffuse, model->light,
			                model->texCoords + (p * 4 + ia) * 4, model->texCoords + (p * 4 + ib) * 4, model->texCoords + (p * 4 + ic) * 4,
			                model->colors + (p * 4 + ia) * 4, model->colors + (p * 4 + ib) * 4, model->colors + (p * 4 + ic) * 4,
			                triangleIndex);
			triangleIndex++;
		}
	}
	free(proj);
	target tg;
	memset(&tg, 0, sizeof(tg));
	tg.color = color; tg.depth = depth; tg.width = desc->width; tg.height = desc->height;
	tg.packOrder = packOrder; tg.stats = stats;
	irect imageBound = {0, 0, desc->width, desc->height};
	if (bands <= 1) {
		row_interval *rows = NULL;
		int32_t capacity = 0;
		for (size_t i = 0; i < commands.count; i++) execute_command(&commands.items[i], &cam, &tg, imageBound, imageBound, &rows, &capacity);
		free(rows);
		if (stats) stats->fragments += tg.fragments;
	} else {
		/* CommandQueue::execute band split (renderCore.cpp:458-479). */
		irect *bandRects = (irect *)malloc(sizeof(irect) * bands);
		int32_t y1 = 0;
		for (int32_t j = 0; j < bands; j++) {
			int32_t y2 = 0 + ((desc->height * (j + 1)) / bands);
			if (j < bands - 1) y2 = (y2 / 2) * 2;
			irect r = {0, y1, desc->width, y2};
			bandRects[j] = r;
			y1 = y2;
		}
		band_job job;
		memset(&job, 0, sizeof(job));
		job.commands = &commands; job.cam = &cam; job.base = tg; job.imageBound = imageBound;
		job.bands = bandRects; job.bandCount = bands;
		pthread_mutex_init(&job.lock, NULL);
		int32_t workers = threads < 1 ? 1 : threads;
		pthread_t *ids = (pthread_t *)malloc(sizeof(pthread_t) * workers);
		for (int32_t w = 0; w < workers; w++) pthread_create(&ids[w], NULL, band_worker, &job);
		for (int32_t w = 0; w < workers; w++) pthread_join(ids[w], NULL);
		pthread_mutex_destroy(&job.lock);
		if (stats) { stats->fragments += job.fragments; stats->trianglesDrawn += job.drawn; }
		free(ids);
		free(bandRects);
	}
	free(commands.items);
	return 0;
}

/* ------------------------------------------------------------------ depth-only */

/* executeTriangleDrawingDepth<AFFINE> (renderCore.cpp:343-387): 1x1 alignment, per-pixel depth += dx. */
static void draw_triangle_depth(const triangle2d *t, const camera *cam, float *depth, int32_t width, int32_t height, irect clipBound,
                                or_stats *stats, uint32_t key, row_interval **rowBuffer, int32_t *rowCapacity) {
	if (!is_frontfacing(t)) return; /* drawTriangleDepth (renderCore.cpp:389-398) */
	if (!rect_overlaps(t->wholeBound, clipBound)) return;
	irect u = rect_cut(t->wholeBound, clipBound);
	irect ab = u;
	ab.top = round_down(u.top, 2);       /* getAlignedRasterBound ignores the alignment arguments */
	ab.bottom = round_up(u.bottom, 2);
	int32_t rowCount = ab.bottom - ab.top;
	if (rowCount <= 0) return;
	if (rowCount > *rowCapacity) {
		*rowBuffer = (row_interval *)realloc(*rowBuffer, sizeof(row_interval) * rowCount);
		*rowCapacity = rowCount;
	}
	row_interval *rows = *rowBuffer;
	rasterize_triangle(t->position[0].flat, t->position[1].flat, t->position[2].flat, rows, ab);
	int affine = !cam->perspective;
	projection proj = get_projection(t, mk3(0.0f, 0.0f, 0.0f), mk3(0.0f, 0.0f, 0.0f), !affine);
	for (int32_t y = ab.top; y < ab.bottom; y++) {
		row_interval row = rows[y - ab.top];
		/* The reference walks the padding row of an odd-height target too, which lies past the end of
		 * its depth image (undefined memory access); the oracle skips that row. */
		if (y >= height) break;
		float value = projection_at(&proj, row.left, y).x;
		float dx = proj.dx.x;
		for (int32_t x = row.left; x < row.right; x++) {
			size_t i = (size_t)y * width + x;
			float old = depth[i];
			if (stats) { stats->fragments++; if (stats->coverage) stats->coverage[i]++; }
			if (affine ? (value < old) : (value > old)) {
				depth[i] = value;
				if (stats && stats->winner) stats->winner[i] = key;
			}
			value += dx;
		}
	}
	if (stats) stats->trianglesDrawn++;
}

/* renderTriangleFromDataDepth (renderCore.cpp:407-443). */
static void render_triangle_depth(const camera *cam, float *depth, int32_t width, int32_t height, projected a, projected b,
                                  projected c, or_stats *stats, uint32_t triangleIndex, row_interval **rows, int32_t *capacity) {
	irect clipBound = {0, 0, width, height};
	triangle2d tri = make_triangle(a, b, c);
	if (triangle_visibility(&tri, cam, 0) == 0) return;
	if (triangle_visibility(&tri, cam, 1) == 1) {
		if (is_frontfacing(&tri)) draw_triangle_depth(&tri, cam, depth, width, height, clipBound, stats, triangleIndex * 8u, rows, capacity);
	} else {
		clipped_triangle ct;
		memset(&ct, 0, sizeof(ct));
		ct.v[0].cs = tri.position[0].cs; ct.v[1].cs = tri.position[1].cs; ct.v[2].cs = tri.position[2].cs;
		ct.v[1].subB = 1.0f; ct.v[2].subC = 1.0f;
		ct.count = 3;
		for (int s = 0; s < cam->clipCount; s++) clipped_clip(&ct, &cam->clip[s]);
		for (int k = 0; k < ct.count - 2; k++) {
			triangle2d sub = make_triangle(camera_to_screen(cam, ct.v[0].cs), camera_to_screen(cam, ct.v[1 + k].cs),
			                               camera_to_screen(cam, ct.v[2 + k].cs));
			draw_triangle_depth(&sub, cam, depth, width, height, clipBound, stats, triangleIndex * 8u + (uint32_t)k, rows, capacity);
		}
	}
}

int or_model_render_depth(const or_model *model, const float modelToWorld[12], const or_camera_desc *desc, float *depth,
                          or_stats *stats) {
	camera cam;
	camera_create(&cam, desc);
	v3 mn, mx;
	model_bound(model, &mn, &mx);
	if (!box_seen(&cam, mn, mx, modelToWorld)) return 0; /* ModelImpl::renderDepth (Model.cpp:199-211) */
	projected *proj = (projected *)malloc(sizeof(projected) * (size_t)(model->pointCount > 0 ? model->pointCount : 1));
	for (int32_t i = 0; i < model->pointCount; i++) {
		v3 p = mk3(model->positions[i * 3], model->positions[i * 3 + 1], model->positions[i * 3 + 2]);
		proj[i] = camera_to_screen(&cam, world_to_camera(&cam, transform_point(modelToWorld, p)));
	}
	row_interval *rows = NULL;
	int32_t capacity = 0;
	uint32_t triangleIndex = 0;
	for (int32_t p = 0; p < model->polyCount; p++) { /* Part::renderDepth (Model.cpp:164-183): quads as (0,1,2), (0,2,3) */
		const int32_t *idx = model->polyIndices + p * 4;
		render_triangle_depth(&cam, depth, desc->width, desc->height, proj[idx[0]], proj[idx[1]], proj[idx[2]], stats, triangleIndex++, &rows, &capacity);
		if (idx[3] >= 0)
			render_triangle_depth(&cam, depth, desc->width, desc->height, proj[idx[0]], proj[idx[2]], proj[idx[3]], stats, triangleIndex++, &rows, &capacity);
	}
	free(rows);
	free(proj);
	return 0;
}

/* ================================================================== deferred light passes */
/* SDK/SpriteEngine (orthoAPI.cpp, lightAPI.cpp) and api/drawAPI.cpp draw_higher, restated
 * for the scalar build (4 lanes per float vector: base/simd.h:4196-4207). */

typedef struct { v3 x, y, z; } m3; /* FMatrix3x3 as axes (math/FMatrix3x3.h:11-30) */

/* normalize (math/FVector.h:113-119): v / length(v), length = sqrtf(squareLength). */
static v3 normalize3(v3 v) {
	float l = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
	if (l == 0.0f) return mk3(0.0f, 0.0f, 1.0f);
	l = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
	return mk3(v.x / l, v.y / l, v.z / l);
}
static v3 cross3(v3 a, v3 b) { return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); } /* FVector.h:101-103 */

/* FMatrix3x3::makeAxisSystem (FMatrix3x3.h:24-30). */
static m3 axis_system(v3 forward, v3 up) {
	m3 r;
	v3 f = normalize3(forward);
	r.z = f;
	r.x = normalize3(cross3(normalize3(up), f));
	r.y = normalize3(cross3(f, r.x));
	return r;
}
static v3 m3_transform(const m3 *m, v3 p) { /* FMatrix3x3.h:31-37 */
	return mk3(p.x * m->x.x + p.y * m->y.x + p.z * m->z.x,
	           p.x * m->x.y + p.y * m->y.y + p.z * m->z.y,
	           p.x * m->x.z + p.y * m->y.z + p.z * m->z.z);
}
static v3 m3_transform_transposed(const m3 *m, v3 p) { /* FMatrix3x3.h:38-44 */
	return mk3(p.x * m->x.x + p.y * m->x.y + p.z * m->x.z,
	           p.x * m->y.x + p.y * m->y.y + p.z * m->y.z,
	           p.x * m->z.x + p.y * m->z.y + p.z * m->z.z);
}
static m3 m3_mul(const m3 *left, const m3 *right) { /* FMatrix3x3.h:50-52 */
	m3 r;
	r.x = m3_transform(right, left->x);
	r.y = m3_transform(right, left->y);
	r.z = m3_transform(right, left->z);
	return r;
}
static m3 m3_inverse(const m3 *m) { /* FMatrix3x3.h:54-80 */
	float det = m->x.x * m->y.y * m->z.z + m->z.x * m->x.y * m->y.z + m->y.x * m->z.y * m->x.z
	          - m->x.x * m->z.y * m->y.z - m->y.x * m->x.y * m->z.z - m->z.x * m->y.y * m->x.z;
	float invDet = 1.0f / det;
	m3 r;
	r.x.x = invDet * (m->y.y * m->z.z - m->y.z * m->z.y);
	r.x.y = -invDet * (m->x.y * m->z.z - m->x.z * m->z.y);
	r.x.z = invDet * (m->x.y * m->y.z - m->x.z * m->y.y);
	r.y.x = -invDet * (m->y.x * m->z.z - m->y.z * m->z.x);
	r.y.y = invDet * (m->x.x * m->z.z - m->x.z * m->z.x);
	r.y.z = -invDet * (m->x.x * m->y.z - m->x.z * m->y.x);
	r.z.x = invDet * (m->y.x * m->z.y - m->y.y * m->z.x);
	r.z.y = -invDet * (m->x.x * m->z.y - m->x.y * m->z.x);
	r.z.z = invDet * (m->x.x * m->y.y - m->x.y * m->y.x);
	return r;
}
static void m3_store(const m3 *m, float *out) {
	out[0] = m->x.x; out[1] = m->x.y; out[2] = m->x.z;
	out[3] = m->y.x; out[4] = m->y.y; out[5] = m->y.z;
	out[6] = m->z.x; out[7] = m->z.y; out[8] = m->z.z;
}
static m3 m3_load(const float *in) {
	m3 m;
	m.x = mk3(in[0], in[1], in[2]); m.y = mk3(in[3], in[4], in[5]); m.z = mk3(in[6], in[7], in[8]);
	return m;
}

/* OrthoView::OrthoView (orthoAPI.cpp:6-37) of OrthoSystem(cameraTilt, pixelsPerTile).view[index]
 * (orthoAPI.cpp:85-123). */
void or_ortho_view_create(float cameraTilt, int32_t pixelsPerTile, int32_t index, or_ortho_view *out) {
	const float diag = 0.707106781f;
	/* sqrt of a float argument resolves to the double overload in the reference's build */
	int32_t yPixelsPerTile = (int32_t)((double)(float)pixelsPerTile / sqrt((double)(cameraTilt * cameraTilt + 1)));
	v3 up = mk3(0.0f, 1.0f, 0.0f);
	v3 forward[8] = {mk3(diag, cameraTilt, diag), mk3(-diag, cameraTilt, diag), mk3(-diag, cameraTilt, -diag),
	                 mk3(diag, cameraTilt, -diag), mk3(0.0f, cameraTilt, 1.0f), mk3(-1.0f, cameraTilt, 0.0f),
	                 mk3(0.0f, cameraTilt, -1.0f), mk3(1.0f, cameraTilt, 0.0f)};
	m3 cameraSystem = axis_system(forward[index], up);
	v3 normalDirection = cameraSystem.z;
	normalDirection.y = 0.0f;
	m3 normalToWorld = axis_system(normalDirection, mk3(0.0f, 1.0f, 0.0f));
	or_camera_desc desc;
	memset(&desc, 0, sizeof(desc));
	desc.location[3] = cameraSystem.x.x; desc.location[4] = cameraSystem.x.y; desc.location[5] = cameraSystem.x.z;
	desc.location[6] = cameraSystem.y.x; desc.location[7] = cameraSystem.y.y; desc.location[8] = cameraSystem.y.z;
	desc.location[9] = cameraSystem.z.x; desc.location[10] = cameraSystem.z.y; desc.location[11] = cameraSystem.z.z;
	desc.perspective = 0;
	desc.slope = 0.5f;
	desc.width = pixelsPerTile;
	desc.height = pixelsPerTile;
	camera cam;
	camera_create(&cam, &desc);
	float halfTile = (float)pixelsPerTile * 0.5f;
	projected px = camera_to_screen(&cam, world_to_camera(&cam, mk3(1.0f, 0.0f, 0.0f)));
	projected pz = camera_to_screen(&cam, world_to_camera(&cam, mk3(0.0f, 0.0f, 1.0f)));
	int32_t xAxis[2] = {(int32_t)(px.is.x - halfTile), (int32_t)(px.is.y - halfTile)};
	int32_t zAxis[2] = {(int32_t)(pz.is.x - halfTile), (int32_t)(pz.is.y - halfTile)};
	m3 tileToScreen;
	tileToScreen.x = mk3((float)xAxis[0], (float)xAxis[1], 0.0f);
	tileToScreen.y = mk3(0.0f, (float)(-yPixelsPerTile), 1.0f);
	tileToScreen.z = mk3((float)zAxis[0], (float)zAxis[1], 0.0f);
	m3 screenToTile = m3_inverse(&tileToScreen);
	m3 toLight;
	toLight.x = m3_transform_transposed(&normalToWorld, screenToTile.x);
	toLight.y = m3_transform_transposed(&normalToWorld, screenToTile.y);
	toLight.z = m3_transform_transposed(&normalToWorld, screenToTile.z);
	m3 fromLight = m3_inverse(&toLight);
	m3_store(&normalToWorld, out->normalToWorld);
	m3_store(&toLight, out->screenDepthToLightSpace);
	m3_store(&fromLight, out->lightSpaceToScreenDepth);
	out->pixelOffsetPerTileX[0] = xAxis[0]; out->pixelOffsetPerTileX[1] = xAxis[1];
	out->pixelOffsetPerTileZ[0] = zAxis[0]; out->pixelOffsetPerTileZ[1] = zAxis[1];
	out->yPixelsPerTile = yPixelsPerTile;
}

/* Camera location of side `side` of a shadow cube map: Transform3D(origin, ShadowCubeMapSides[side] *
 * normalToWorld) (SDK/SpriteEngine/spriteAPI.cpp:328-336, 377-381). */
void or_shadow_side_location(const float normalToWorld[9], int32_t side, float location[12]) {
	v3 forward[6] = {mk3(1.0f, 0.0f, 0.0f), mk3(-1.0f, 0.0f, 0.0f), mk3(0.0f, 1.0f, 0.0f),
	                 mk3(0.0f, -1.0f, 0.0f), mk3(0.0f, 0.0f, 1.0f), mk3(0.0f, 0.0f, -1.0f)};
	v3 up[6] = {mk3(0.0f, 1.0f, 0.0f), mk3(0.0f, 1.0f, 0.0f), mk3(0.0f, 0.0f, 1.0f),
	            mk3(0.0f, 0.0f, 1.0f), mk3(0.0f, 1.0f, 0.0f), mk3(0.0f, 1.0f, 0.0f)};
	m3 s = axis_system(forward[side], up[side]);
	m3 n = m3_load(normalToWorld);
	m3 r = m3_mul(&s, &n);
	location[0] = 0.0f; location[1] = 0.0f; location[2] = 0.0f;
	m3_store(&r, location + 3);
}

static inline uint32_t sat_add_bytes(uint32_t a, uint32_t b) { /* saturatedAddition of U8 lanes (base/simd.h:2670-2690) */
	uint32_t out = 0;
	for (int i = 0; i < 4; i++) {
		uint32_t s = ((a >> (8 * i)) & 0xFFu) + ((b >> (8 * i)) & 0xFFu);
		out |= (s > 255u ? 255u : s) << (8 * i);
	}
	return out;
}
static inline float vmin_ref(float left, float right) { return (right < left) ? right : left; } /* simd.h:2198-2216 */
static inline float vmax_ref(float left, float right) { return (right > left) ? right : left; } /* simd.h:2217-2235 */
/* reciprocalSquareRoot of the scalar build (simd.h:4084-4104): 1.0f / sqrt(x) through the double overload. */
static inline float rsqrt_ref(float x) { return (float)(1.0 / sqrt((double)x)); }
static inline float sqrt_ref(float x) { return (float)sqrt((double)x); } /* squareRoot (simd.h:4130-4146) */
static inline uint32_t light_bytes(float r, float g, float b) { /* packOrder_packBytes(r, g, b) of truncated, clamped channels */
	return trunc_u32(vmin_ref(r, 255.1f)) | (trunc_u32(vmin_ref(g, 255.1f)) << 8) | (trunc_u32(vmin_ref(b, 255.1f)) << 16);
}

/* setDirectedLight / addDirectedLight (lightAPI.cpp:23-74). */
void or_directed_light(const or_ortho_view *view, uint32_t *light, int32_t lightStride, const uint32_t *normal,
                       int32_t normalStride, int32_t width, int32_t height, const float direction[3], float intensity,
                       const int32_t color[3], int32_t add) {
	m3 n = m3_load(view->normalToWorld);
	v3 d = normalize3(m3_transform_transposed(&n, mk3(direction[0], direction[1], direction[2])));
	v3 rev = mk3(-d.x, -d.y, -d.z);
	rev = scale3(rev, intensity);
	rev = scale3(rev, 2.0f);
	float cr = fmaxf_ref(0.0f, (float)color[0] / 255.0f), cg = fmaxf_ref(0.0f, (float)color[1] / 255.0f);
	float cb = fmaxf_ref(0.0f, (float)color[2] / 255.0f);
	for (int32_t y = 0; y < height; y++) {
		for (int32_t x = 0; x < width; x++) {
			uint32_t c = normal[(size_t)y * normalStride + x];
			v3 neg = mk3((float)(c & 0xFFu) - 128.0f, (float)((c >> 8) & 0xFFu) - 128.0f, (float)((c >> 16) & 0xFFu) - 128.0f);
			float i = vmax_ref(0.0f, dot3(neg, rev));
			uint32_t bytes = light_bytes(i * cr, i * cg, i * cb);
			uint32_t *p = light + (size_t)y * lightStride + x;
			*p = add ? sat_add_bytes(*p, bytes) : bytes;
		}
	}
}

/* getShadowTransparency (lightAPI.cpp:104-138). */
static float shadow_transparency(const float *cube, int32_t width, float halfWidth, v3 o) {
	float absX = o.x < 0.0f ? -o.x : o.x, absY = o.y < 0.0f ? -o.y : o.y, absZ = o.z < 0.0f ? -o.z : o.z;
	int xIsLongest = absX > absY && absX > absZ;
	int yIsLongerThanZ = absY > absZ;
	float depth = xIsLongest ? o.x : (yIsLongerThanZ ? o.y : o.z);
	float slopeUp = (yIsLongerThanZ && !xIsLongest) ? o.z : o.y;
	float slopeSide = xIsLongest ? -o.z : (yIsLongerThanZ ? -o.x : o.x);
	int32_t viewOffset = width * (xIsLongest ? 0 : (yIsLongerThanZ ? 2 : 4));
	int negativeSide = depth < 0.0f;
	if (negativeSide) { depth = -depth; slopeSide = -slopeSide; viewOffset = viewOffset + width; }
	float reciDepth = 1.0f / depth;
	float scale = halfWidth * reciDepth;
	int32_t sampleX = (int32_t)(halfWidth + (slopeSide * scale));
	int32_t sampleY = (int32_t)(halfWidth - (slopeUp * scale));
	int32_t maxPixel = width - 1;
	if (sampleX < 0) sampleX = 0;
	if (sampleX > maxPixel) sampleX = maxPixel;
	if (sampleY < 0) sampleY = 0;
	if (sampleY > maxPixel) sampleY = maxPixel;
	float shadowReciDepth = cube[((sampleY + viewOffset) * width) + sampleX];
	return reciDepth * 1.02f > shadowReciDepth ? 1.0f : 0.0f;
}

/* calculateBound (lightAPI.cpp:76-102) with alignment 4; returns 0 when nothing is lit. */
int32_t or_point_light_bound(const or_ortho_view *view, int32_t centerX, int32_t centerY, int32_t width, int32_t height,
                             const float position[3], float radius, int32_t bound[4]) {
	m3 n = m3_load(view->normalToWorld), fromLight = m3_load(view->lightSpaceToScreenDepth);
	v3 lightSpace = m3_transform_transposed(&n, mk3(position[0], position[1], position[2]));
	v3 rotated = m3_transform(&fromLight, lightSpace);
	int32_t pcx = (int32_t)rotated.x + centerX, pcy = (int32_t)rotated.y + centerY;
	int32_t pixelRadius = (int32_t)(radius * fromLight.x.x);
	if (pcx < -pixelRadius || pcx > width + pixelRadius || pcy < -pixelRadius || pcy > height + pixelRadius) return 0;
	irect image = {0, 0, width, height};
	int32_t side = (int32_t)((float)pixelRadius * 2.0f);
	irect light = {pcx - pixelRadius, pcy - pixelRadius, pcx - pixelRadius + side, pcy - pixelRadius + side};
	irect r = rect_cut(image, light);
	if (!(r.right - r.left > 0 && r.bottom - r.top > 0)) return 0;
	bound[0] = round_down(r.left, 4); bound[1] = r.top; bound[2] = round_up(r.right, 4); bound[3] = r.bottom;
	return 1;
}

/* addPointLight (lightAPI.cpp:169-285).  Rows are split into the bands of threadedSplit
 * (base/threading.cpp:193-263) for `threads` hardware threads: each band restarts the
 * light-space sweep from its own top row. */
void or_point_light(const or_ortho_view *view, int32_t centerX, int32_t centerY, uint32_t *light, int32_t lightStride,
                    const uint32_t *normal, int32_t normalStride, const float *heightImage, int32_t heightStride,
                    int32_t width, int32_t height, const float position[3], float radius, float intensity,
                    const int32_t color[3], const float *shadowCube, int32_t cubeWidth, int32_t threads) {
	int32_t b[4];
	if (!or_point_light_bound(view, centerX, centerY, width, height, position, radius, b)) return;
	m3 n = m3_load(view->normalToWorld), toLight = m3_load(view->screenDepthToLightSpace);
	v3 source = m3_transform_transposed(&n, mk3(position[0], position[1], position[2]));
	v3 face = toLight.z;
	float cr = fmaxf_ref(0.0f, (float)color[0] * intensity), cg = fmaxf_ref(0.0f, (float)color[1] * intensity);
	float cb = fmaxf_ref(0.0f, (float)color[2] * intensity);
	float reciprocalRadius = 1.0f / radius;
	float cubeCenter = (float)cubeWidth * 0.5f;
	int32_t rows = b[3] - b[1];
	int32_t jobs = (threads > 0 ? threads : 1) * 2;
	if (jobs > rows / 128) jobs = rows / 128;
	if (jobs < 1) jobs = 1;
	v3 dx = toLight.x, dy = toLight.y;
	v3 dxX = scale3(dx, 4.0f);
	for (int32_t job = 0; job < jobs; job++) {
		int32_t y1 = job == 0 ? b[1] : (job * rows) / jobs + b[1];
		int32_t y2 = job + 1 >= jobs ? b[3] : ((job + 1) * rows) / jobs + b[1];
		v3 base = sub3(m3_transform(&toLight, mk3(0.5f - (float)centerX + (float)b[0], 0.5f - (float)centerY + (float)y1, 0.0f)), source);
		v3 lane[4]; /* F32xXx3::createGradient (base/simd.h:474-476, simd3D.h:211-216) */
		lane[0] = base;
		lane[1] = mk3(base.x + dx.x, base.y + dx.y, base.z + dx.z);
		lane[2] = mk3(base.x + dx.x * 2.0f, base.y + dx.y * 2.0f, base.z + dx.z * 2.0f);
		lane[3] = mk3(base.x + dx.x * 3.0f, base.y + dx.y * 3.0f, base.z + dx.z * 3.0f);
		for (int32_t y = y1; y < y2; y++) {
			v3 pixel[4] = {lane[0], lane[1], lane[2], lane[3]};
			for (int32_t x = b[0]; x < b[2]; x += 4) {
				for (int l = 0; l < 4; l++) {
					int32_t xx = x + l;
					if (xx < width) {
						float depth = heightImage[(size_t)y * heightStride + xx];
						v3 o = mk3(pixel[l].x + face.x * depth, pixel[l].y + face.y * depth, pixel[l].z + face.z * depth);
						float squareLength = (o.x * o.x + o.y * o.y) + o.z * o.z;
						float ratio = vmin_ref(1.0f, sqrt_ref(squareLength) * reciprocalRadius);
						uint32_t nc = normal[(size_t)y * normalStride + xx];
						v3 neg = mk3(((float)(nc & 0xFFu) - 128.0f) * (-1.0f / 128.0f),
						             ((float)((nc >> 8) & 0xFFu) - 128.0f) * (-1.0f / 128.0f),
						             ((float)((nc >> 16) & 0xFFu) - 128.0f) * (-1.0f / 128.0f));
						float distanceIntensity = 1.0f - 2.0f * ratio + ratio * ratio;
						float rs = rsqrt_ref(squareLength);
						v3 unit = mk3(o.x * rs, o.y * rs, o.z * rs);
						float angle = vmax_ref(0.0f, (unit.x * neg.x + unit.y * neg.y) + unit.z * neg.z);
						float i = angle * distanceIntensity;
						if (shadowCube) i = i * shadow_transparency(shadowCube, cubeWidth, cubeCenter, o);
						uint32_t *p = light + (size_t)y * lightStride + xx;
						*p = sat_add_bytes(*p, light_bytes(i * cr, i * cg, i * cb));
					}
					pixel[l] = add3(pixel[l], dxX);
				}
			}
			for (int l = 0; l < 4; l++) lane[l] = add3(lane[l], dy);
		}
	}
}

/* blendLight (lightAPI.cpp:287-323). */
void or_blend_light(uint32_t *target, int32_t targetStride, int32_t targetPackOrder, const uint32_t *diffuse,
                    int32_t diffuseStride, const uint32_t *lightImage, int32_t lightStride, int32_t width, int32_t height) {
	static const uint32_t shifts[4][3] = {{0, 8, 16}, {16, 8, 0}, {8, 16, 24}, {24, 16, 8}}; /* image/PackOrder.h:80-92 */
	const float scale = (float)(1.0 / 128.0f);
	for (int32_t y = 0; y < height; y++) {
		for (int32_t x = 0; x < width; x++) {
			uint32_t d = diffuse[(size_t)y * diffuseStride + x], l = lightImage[(size_t)y * lightStride + x];
			uint32_t out = 0;
			for (int ch = 0; ch < 3; ch++) {
				float v = ((float)((d >> (8 * ch)) & 0xFFu) * (float)((l >> (8 * ch)) & 0xFFu)) * scale;
				out |= trunc_u32(vmin_ref(v, 255.1f)) << shifts[targetPackOrder][ch];
			}
			target[(size_t)y * targetStride + x] = out;
		}
	}
}

/* Byte index of red, green, blue, alpha in memory for a PackOrderIndex (image/PackOrder.h:61-92). */
static void pack_indices(int32_t order, int idx[4]) {
	static const int table[4][4] = {{0, 1, 2, 3}, {2, 1, 0, 3}, {1, 2, 3, 0}, {3, 2, 1, 0}};
	for (int i = 0; i < 4; i++) idx[i] = table[order][i];
}

/* draw_higher with two colour images (api/drawAPI.cpp:872-900, 946-981): every source pixel above
 * -inf, raised by offset, replaces the target height and both colours when strictly higher. */
void or_draw_higher(float *targetHeight, int32_t thStride, uint32_t *targetA, int32_t taStride, int32_t taPack,
                    uint32_t *targetB, int32_t tbStride, int32_t tbPack, int32_t tw, int32_t th, const float *sourceHeight,
                    int32_t shStride, const uint32_t *sourceA, int32_t saStride, int32_t saPack, const uint32_t *sourceB,
                    int32_t sbStride, int32_t sbPack, int32_t sw, int32_t sh, int32_t left, int32_t top, float offset) {
	int ta[4], tb[4], sa[4], sb[4];
	pack_indices(taPack, ta); pack_indices(tbPack, tb); pack_indices(saPack, sa); pack_indices(sbPack, sb);
	int32_t x0 = left > 0 ? left : 0, y0 = top > 0 ? top : 0;
	int32_t x1 = left + sw < tw ? left + sw : tw, y1 = top + sh < th ? top + sh : th;
	for (int32_t y = y0; y < y1; y++) {
		for (int32_t x = x0; x < x1; x++) {
			int32_t sx = x - left, sy = y - top;
			float h = sourceHeight[(size_t)sy * shStride + sx];
			if (h > -INFINITY) {
				h += offset;
				float *t = targetHeight + (size_t)y * thStride + x;
				if (h > *t) {
					*t = h;
					const uint8_t *pa = (const uint8_t *)(sourceA + (size_t)sy * saStride + sx);
					const uint8_t *pb = (const uint8_t *)(sourceB + (size_t)sy * sbStride + sx);
					uint8_t *qa = (uint8_t *)(targetA + (size_t)y * taStride + x);
					uint8_t *qb = (uint8_t *)(targetB + (size_t)y * tbStride + x);
					for (int c = 0; c < 4; c++) { qa[ta[c]] = pa[sa[c]]; qb[tb[c]] = pb[sb[c]]; }
				}
			}
		}
	}
}

/* ------------------------------------------------------------------ renderer with an occlusion grid */

/* RendererImpl (api/rendererAPI.cpp:141-477): renderer_begin / renderer_giveTask / the occlusion
 * grid (occludeFromBox, occludeFromTopRows, occludeFromExistingTriangles, isBoxVisible,
 * completeOcclusion) / renderer_end.  The grid holds, per 16x16 cell, the largest camera-space
 * depth at which something may still be visible; commands whose nearest corner is behind it are
 * not drawn.  Commands are executed in one band (the band split does not change the result). */
#define OR_CELL 16

typedef struct { int32_t x1, y1, x2, y2; uint32_t color; } debug_line; /* DebugLine (rendererAPI.cpp:132-137), colour as RGBA bytes */

/* drawLineSuper (api/drawAPI.cpp:176-279) of a packed colour: horizontal and vertical runs, else
 * the reference's integer error walk along the longer axis; only pixels inside the image are written. */
static void draw_line(uint32_t *image, int32_t width, int32_t height, int32_t x1, int32_t y1, int32_t x2, int32_t y2, uint32_t color) {
	if ((x1 < 0 && x2 < 0) || (y1 < 0 && y2 < 0) || (x1 >= width && x2 >= width) || (y1 >= height && y2 >= height)) return;
#define PUT(X, Y) do { int32_t px_ = (X), py_ = (Y); if (px_ >= 0 && py_ >= 0 && px_ < width && py_ < height) image[(size_t)py_ * width + px_] = color; } while (0)
	if (y1 == y2) {
		int32_t l = x1 < x2 ? x1 : x2, r = x1 < x2 ? x2 : x1;
		for (int32_t x = l; x <= r; x++) PUT(x, y1);
	} else if (x1 == x2) {
		int32_t t = y1 < y2 ? y1 : y2, b = y1 < y2 ? y2 : y1;
		for (int32_t y = t; y <= b; y++) PUT(x1, y);
	} else {
		int32_t adx = x2 > x1 ? x2 - x1 : x1 - x2, ady = y2 > y1 ? y2 - y1 : y1 - y2;
		if (ady >= adx) {
			if (y2 < y1) { int32_t t = x1; x1 = x2; x2 = t; t = y1; y1 = y2; y2 = t; }
			int32_t step = x2 > x1 ? 1 : -1, tilt = (x2 > x1 ? x2 - x1 : x1 - x2) * 2, maxError = y2 - y1, error = 0, x = x1;
			for (int32_t y = y1; y <= y2; y++) {
				PUT(x, y);
				error += tilt;
				if (error >= maxError) { x += step; error -= maxError * 2; }
			}
		} else {
			if (x2 < x1) { int32_t t = x1; x1 = x2; x2 = t; t = y1; y1 = y2; y2 = t; }
			int32_t step = y2 > y1 ? 1 : -1, tilt = (y2 > y1 ? y2 - y1 : y1 - y2) * 2, maxError = x2 - x1, error = 0, y = y1;
			for (int32_t x = x1; x <= x2; x++) {
				PUT(x, y);
				error += tilt;
				if (error >= maxError) { y += step; error -= maxError * 2; }
			}
		}
	}
#undef PUT
}

void or_draw_line(uint32_t *image, int32_t width, int32_t height, int32_t x1, int32_t y1, int32_t x2, int32_t y2, uint32_t color) {
	draw_line(image, width, height, x1, y1, x2, y2, color);
}

struct or_renderer_s {
	int receiving;
	uint32_t *color;
	float *depth;
	int32_t width, height, packOrder;
	command_list commands;
	camera *cams;
	int32_t camCount, camCapacity;
	uint32_t triangles;
	float *grid;
	int32_t gridAllocWidth, gridAllocHeight; /* the allocated grid (its stride is gridAllocWidth) */
	int32_t gridWidth, gridHeight;
	int occluded;
	debug_line *debugLines;
	int32_t debugCount, debugCapacity;
};

or_renderer *or_renderer_create(void) { return (or_renderer *)calloc(1, sizeof(or_renderer)); }

void or_renderer_destroy(or_renderer *r) {
	if (!r) return;
	free(r->commands.items);
	free(r->cams);
	free(r->grid);
	free(r->debugLines);
	free(r);
}

int or_renderer_begin(or_renderer *r, uint32_t *color, float *depth, int32_t width, int32_t height, int32_t packOrder) {
	if (r->receiving) return -1;
	r->receiving = 1;
	r->color = color;
	r->depth = depth;
	r->width = width;
	r->height = height;
	r->packOrder = packOrder;
	r->gridWidth = (width + (OR_CELL - 1)) / OR_CELL;
	r->gridHeight = (height + (OR_CELL - 1)) / OR_CELL;
	r->occluded = 0;
	r->commands.count = 0;
	r->camCount = 0;
	r->triangles = 0;
	return 0;
}

/* getOuterCellBound (rendererAPI.cpp:168-179). */
static irect outer_cell_bound(const or_renderer *r, irect pixelBound) {
	int32_t minX = pixelBound.left / OR_CELL, maxX = pixelBound.right / OR_CELL + 1;
	int32_t minY = pixelBound.top / OR_CELL, maxY = pixelBound.bottom / OR_CELL + 1;
	if (minX < 0) minX = 0;
	if (minY < 0) minY = 0;
	if (maxX > r->gridWidth) maxX = r->gridWidth;
	if (maxY > r->gridHeight) maxY = r->gridHeight;
	irect out = {minX, minY, maxX, maxY};
	return out;
}

static float *grid_cell(const or_renderer *r, int32_t x, int32_t y) { return r->grid + (size_t)y * r->gridAllocWidth + x; }

/* image_readPixel_clamp (api/imageAPI.h:276-282) of the grid image: 0 while no grid exists, and
 * clamped to the allocated grid, which may be another frame's. */
static float grid_read(const or_renderer *r, int32_t x, int32_t y) {
	if (!r->grid || r->gridAllocWidth <= 0 || r->gridAllocHeight <= 0) return 0.0f;
	if (x < 0) x = 0;
	if (y < 0) y = 0;
	if (x > r->gridAllocWidth - 1) x = r->gridAllocWidth - 1;
	if (y > r->gridAllocHeight - 1) y = r->gridAllocHeight - 1;
	return *grid_cell(r, x, y);
}

/* prepareForOcclusion (rendererAPI.cpp:181-191). */
static void prepare_for_occlusion(or_renderer *r) {
	if (!r->occluded) {
		if (!(r->grid && r->gridAllocWidth >= r->gridWidth && r->gridAllocHeight >= r->gridHeight)) {
			free(r->grid);
			r->gridAllocWidth = r->gridWidth;
			r->gridAllocHeight = r->gridHeight;
			r->grid = (float *)malloc(sizeof(float) * (size_t)(r->gridWidth > 0 ? r->gridWidth : 1) * (size_t)(r->gridHeight > 0 ? r->gridHeight : 1));
		}
		for (size_t i = 0; i < (size_t)r->gridAllocWidth * (size_t)r->gridAllocHeight; i++) r->grid[i] = INFINITY;
	}
	r->occluded = 1;
}

/* pointInsideOfEdge / pointInsideOfHull / rectangleInsideOfHull (rendererAPI.cpp:100-130). */
static int point_inside_hull(const projected *hull, int32_t count, int64_t px, int64_t py) {
	for (int32_t c = 0; c < count; c++) {
		int32_t nc = c + 1;
		if (nc == count) nc = 0;
		int64_t ex = hull[nc].flat.y - hull[c].flat.y, ey = hull[c].flat.x - hull[nc].flat.x;
		int64_t rx = px - hull[c].flat.x, ry = py - hull[c].flat.y;
		if (!(ex * rx + ey * ry <= 0)) return 0;
	}
	return 1;
}

/* occludeFromSortedHull (rendererAPI.cpp:216-239). */
static void occlude_from_sorted_hull(or_renderer *r, const projected *hull, int32_t count, irect pixelBound) {
	if ((pixelBound.right - pixelBound.left) > OR_CELL && (pixelBound.bottom - pixelBound.top) > OR_CELL) {
		float distance = 0.0f;
		for (int32_t c = 0; c < count; c++) if (hull[c].cs.z > distance) distance = hull[c].cs.z;
		irect cells = outer_cell_bound(r, pixelBound);
		for (int32_t cy = cells.top; cy < cells.bottom; cy++) {
			for (int32_t cx = cells.left; cx < cells.right; cx++) {
				int64_t left = (int64_t)(cx * OR_CELL * 256), top = (int64_t)(cy * OR_CELL * 256);
				int64_t right = left + OR_CELL * 256, bottom = top + OR_CELL * 256;
				if (point_inside_hull(hull, count, left, top) && point_inside_hull(hull, count, right, top) &&
				    point_inside_hull(hull, count, left, bottom) && point_inside_hull(hull, count, right, bottom)) {
					if (distance < grid_read(r, cx, cy)) *grid_cell(r, cx, cy) = distance;
				}
			}
		}
	}
}

/* getPixelBoundFromProjection (rendererAPI.cpp:92-98). */
static irect pixel_bound_of(const projected *points, int32_t count) {
	irect b;
	b.left = (int32_t)(points[0].flat.x / 256); b.top = (int32_t)(points[0].flat.y / 256);
	b.right = b.left + 1; b.bottom = b.top + 1;
	for (int32_t p = 1; p < count; p++) {
		int32_t x = (int32_t)(points[p].flat.x / 256), y = (int32_t)(points[p].flat.y / 256);
		if (x < b.left) b.left = x;
		if (y < b.top) b.top = y;
		if (x + 1 > b.right) b.right = x + 1;
		if (y + 1 > b.bottom) b.bottom = y + 1;
	}
	return b;
}

/* jarvisConvexHullAlgorithm (rendererAPI.cpp:38-72). */
static int counter_clockwise(const projected *p, const projected *q, const projected *s) {
	return (q->flat.y - p->flat.y) * (s->flat.x - q->flat.x) - (q->flat.x - p->flat.x) * (s->flat.y - q->flat.y) < 0;
}
static void jarvis_hull(projected *out, int32_t *outCount, const projected *in, int32_t n) {
	if (n < 3) {
		*outCount = n;
		for (int32_t p = 0; p < n; p++) out[p] = in[p];
		return;
	}
	int32_t l = 0;
	*outCount = 0;
	for (int32_t i = 1; i < n; i++) if (in[i].flat.x < in[l].flat.x) l = i;
	int32_t p = l;
	do {
		if (*outCount >= n) return;
		out[(*outCount)++] = in[p];
		int32_t q = (p + 1) % n;
		for (int32_t i = 0; i < n; i++) if (counter_clockwise(&in[p], &in[i], &in[q])) q = i;
		p = q;
	} while (p != l);
}

static void box_corners(const float mn[3], const float mx[3], v3 out[8]) { /* GENERATE_BOX_CORNERS (rendererAPI.cpp:257-265) */
	out[0] = mk3(mn[0], mn[1], mn[2]); out[1] = mk3(mn[0], mn[1], mx[2]);
	out[2] = mk3(mn[0], mx[1], mn[2]); out[3] = mk3(mn[0], mx[1], mx[2]);
	out[4] = mk3(mx[0], mn[1], mn[2]); out[5] = mk3(mx[0], mn[1], mx[2]);
	out[6] = mk3(mx[0], mx[1], mn[2]); out[7] = mk3(mx[0], mx[1], mx[2]);
}

static void push_debug_line(or_renderer *r, int32_t x1, int32_t y1, int32_t x2, int32_t y2, uint32_t color) {
	if (r->debugCount == r->debugCapacity) {
		r->debugCapacity = r->debugCapacity ? r->debugCapacity * 2 : 64;
		r->debugLines = (debug_line *)realloc(r->debugLines, sizeof(debug_line) * (size_t)r->debugCapacity);
	}
	debug_line l = {x1, y1, x2, y2, color};
	r->debugLines[r->debugCount++] = l;
}

int or_renderer_occlude_from_box(or_renderer *r, const float mn[3], const float mx[3], const float modelToWorld[12],
                                 const or_camera_desc *desc, int debugSilhouette) {
	if (!r->receiving) return -1;
	prepare_for_occlusion(r);
	camera cam;
	camera_create(&cam, desc);
	v3 local[8];
	box_corners(mn, mx, local);
	projected proj[8], hull[8];
	for (int p = 0; p < 8; p++) { /* projectHull (rendererAPI.cpp:76-90) */
		v3 cs = world_to_camera(&cam, transform_point(modelToWorld, local[p]));
		v3 narrow = mk3(cs.x * 0.5f, cs.y * 0.5f, cs.z * 1.0f);
		for (int s = 0; s < cam.cullCount; s++)
			if (!plane_inside(&cam.cull[s], narrow)) return 0;
		proj[p] = camera_to_screen(&cam, cs);
	}
	int32_t count = 0;
	jarvis_hull(hull, &count, proj, 8);
	occlude_from_sorted_hull(r, hull, count, pixel_bound_of(hull, count));
	if (debugSilhouette) {
		/* cyan lines around the hull, kept until renderer_end; the reference tests the depth of
		 * projections[p] (unsorted), not of the hull corner it draws from (rendererAPI.cpp:277-291) */
		for (int32_t p = 0; p < count; p++) {
			int32_t q = (p + 1) % count;
			if (proj[p].cs.z > cam.nearClip)
				push_debug_line(r, (int32_t)(hull[p].flat.x / 256), (int32_t)(hull[p].flat.y / 256), (int32_t)(hull[q].flat.x / 256),
				                (int32_t)(hull[q].flat.y / 256), 0xFFFFFF00u /* red 0, green, blue, alpha 255 */);
		}
	}
	return 0;
}

int or_renderer_occlude_from_existing_triangles(or_renderer *r) {
	if (!r->receiving) return -1;
	prepare_for_occlusion(r);
	for (size_t t = 0; t < r->commands.count; t++) {
		const command *c = &r->commands.items[t];
		if (c->filter == 0) occlude_from_sorted_hull(r, c->triangle.position, 3, c->triangle.wholeBound);
	}
	return 0;
}

/* occludeFromTopRows (rendererAPI.cpp:417-476): the top pixel row of each cell row, in cell-wide
 * runs that start one pixel early after the first. */
int or_renderer_occlude_from_top_rows(or_renderer *r, int perspective) {
	prepare_for_occlusion(r);
	if (!r->receiving) return -1;
	if (!r->depth) return -2;
	for (int32_t gy = 0; gy < r->gridHeight; gy++) {
		const float *row = r->depth + (size_t)(gy * OR_CELL) * r->width;
		int32_t x = 0, right = OR_CELL - 1;
		for (int32_t gx = 0; gx < r->gridWidth; gx++) {
			if (right >= r->width) right = r->width;
			float value;
			if (perspective) {
				float maxInv = INFINITY;
				while (x < right) { if (row[x] < maxInv) maxInv = row[x]; x++; }
				value = 1.0f / maxInv;
			} else {
				value = 0.0f;
				while (x < right) { if (row[x] > value) value = row[x]; x++; }
			}
			if (value < *grid_cell(r, gx, gy)) *grid_cell(r, gx, gy) = value;
			right += OR_CELL;
		}
	}
	return 0;
}

/* isHullOccluded / isBoxOccluded (rendererAPI.cpp:297-341); returns 1 when visible. */
int or_renderer_is_box_visible(const or_renderer *r, const float mn[3], const float mx[3], const float modelToWorld[12],
                               const or_camera_desc *desc) {
	camera cam;
	camera_create(&cam, desc);
	v3 local[8], cs[8];
	projected proj[8];
	box_corners(mn, mx, local);
	for (int p = 0; p < 8; p++) {
		cs[p] = world_to_camera(&cam, transform_point(modelToWorld, local[p]));
		proj[p] = camera_to_screen(&cam, cs[p]);
	}
	for (int s = 0; s < cam.cullCount; s++) {
		int allOutside = 1;
		for (int p = 0; p < 8; p++) if (plane_inside(&cam.cull[s], cs[p])) { allOutside = 0; break; }
		if (allOutside) return 0;
	}
	irect pixelBound = pixel_bound_of(proj, 8);
	float closest = INFINITY;
	for (int p = 0; p < 8; p++) if (proj[p].cs.z < closest) closest = proj[p].cs.z;
	irect cells = outer_cell_bound(r, pixelBound);
	for (int32_t cy = cells.top; cy < cells.bottom; cy++)
		for (int32_t cx = cells.left; cx < cells.right; cx++)
			if (closest < grid_read(r, cx, cy)) return 1;
	return 0;
}

int or_renderer_has_occluders(const or_renderer *r) { return r->occluded; }

/* model_render_threaded (modelAPI.cpp:214-275): culling, occlusion of the whole model, then one
 * renderer_giveTask_triangle per fan triangle. */
int or_renderer_give_task(or_renderer *r, const or_model *model, const float modelToWorld[12], const or_camera_desc *desc) {
	if (!r->receiving) return -1;
	camera cam;
	camera_create(&cam, desc);
	v3 mn, mx;
	model_bound(model, &mn, &mx);
	if (!box_seen(&cam, mn, mx, modelToWorld)) return 0;
	if (r->occluded) {
		const float bmn[3] = {mn.x, mn.y, mn.z}, bmx[3] = {mx.x, mx.y, mx.z};
		if (!or_renderer_is_box_visible(r, bmn, bmx, modelToWorld, desc)) return 0;
	}
	if (r->camCount == r->camCapacity) {
		r->camCapacity = r->camCapacity ? r->camCapacity * 2 : 16;
		r->cams = (camera *)realloc(r->cams, sizeof(camera) * (size_t)r->camCapacity);
	}
	const int32_t taskIndex = r->camCount++;
	r->cams[taskIndex] = cam;
	projected *proj = (projected *)malloc(sizeof(projected) * (size_t)(model->pointCount > 0 ? model->pointCount : 1));
	for (int32_t i = 0; i < model->pointCount; i++) {
		v3 p = mk3(model->positions[i * 3], model->positions[i * 3 + 1], model->positions[i * 3 + 2]);
		proj[i] = camera_to_screen(&cam, world_to_camera(&cam, transform_point(modelToWorld, p)));
	}
	const size_t before = r->commands.count;
	for (int32_t p = 0; p < model->polyCount; p++) {
		const int32_t *idx = model->polyIndices + p * 4;
		int triCount = (idx[3] < 0) ? 1 : 2;
		for (int t = 0; t < triCount; t++) {
			int ia = 0, ib = 1 + t, ic = 2 + t;
			submit_triangle(&r->commands, &cam, r->color != NULL, r->depth != NULL, r->width, r->height,
			                proj[idx[ia]], proj[idx[ib]], proj[idx[ic]], model->filter, model->diffuse, model->light,
			                model->texCoords + (p * 4 + ia) * 4, model->texCoords + (p * 4 + ib) * 4, model->texCoords + (p * 4 + ic) * 4,
			                model->colors + (p * 4 + ia) * 4, model->colors + (p * 4 + ib) * 4, model->colors + (p * 4 + ic) * 4,
			                r->triangles);
			r->triangles++;
		}
	}
	for (size_t i = before; i < r->commands.count; i++) { r->commands.items[i].task = taskIndex; r->commands.items[i].occluded = 0; }
	free(proj);
	return 0;
}

/* renderer_giveTask_triangle (rendererAPI.cpp:503-519): renderTriangleFromData of corners given
 * projected; corner k of the triangle: cs (3 floats), is (2 floats), flat (2 int64). */
int or_renderer_give_triangle(or_renderer *r, const float cs[9], const float is[6], const int64_t flat[6], const float colors[12],
                              const float texCoords[12], const or_texture *diffuse, const or_texture *light, int filter,
                              const or_camera_desc *desc) {
	if (!r->receiving) return -1;
	if (r->camCount == r->camCapacity) {
		r->camCapacity = r->camCapacity ? r->camCapacity * 2 : 16;
		r->cams = (camera *)realloc(r->cams, sizeof(camera) * (size_t)r->camCapacity);
	}
	const int32_t taskIndex = r->camCount++;
	camera_create(&r->cams[taskIndex], desc);
	projected p[3];
	for (int k = 0; k < 3; k++) {
		p[k].cs = mk3(cs[3 * k], cs[3 * k + 1], cs[3 * k + 2]);
		p[k].is.x = is[2 * k]; p[k].is.y = is[2 * k + 1];
		p[k].flat.x = flat[2 * k]; p[k].flat.y = flat[2 * k + 1];
	}
	const size_t before = r->commands.count;
	submit_triangle(&r->commands, &r->cams[taskIndex], r->color != NULL, r->depth != NULL, r->width, r->height, p[0], p[1], p[2],
	                filter, diffuse, light, texCoords, texCoords + 4, texCoords + 8, colors, colors + 4, colors + 8, r->triangles);
	r->triangles++;
	for (size_t i = before; i < r->commands.count; i++) { r->commands.items[i].task = taskIndex; r->commands.items[i].occluded = 0; }
	return 0;
}

/* completeOcclusion (rendererAPI.cpp:193-214), CommandQueue::execute of the commands left, then the
 * debug overlays of endFrame (rendererAPI.cpp:354-415): white lines around every drawn command
 * when debugWireframe, then the silhouettes kept by occludeFromBox. */
int or_renderer_end(or_renderer *r, or_stats *stats, int debugWireframe) {
	if (!r->receiving) return -1;
	r->receiving = 0;
	if (r->occluded) {
		for (size_t t = 0; t < r->commands.count; t++) {
			command *c = &r->commands.items[t];
			irect cells = outer_cell_bound(r, c->triangle.wholeBound);
			float depth = c->triangle.position[0].cs.z;
			if (c->triangle.position[1].cs.z < depth) depth = c->triangle.position[1].cs.z;
			if (c->triangle.position[2].cs.z < depth) depth = c->triangle.position[2].cs.z;
			int anyVisible = 0;
			for (int32_t cy = cells.top; cy < cells.bottom; cy++)
				for (int32_t cx = cells.left; cx < cells.right; cx++)
					if ((double)depth < (double)grid_read(r, cx, cy) + 0.001) anyVisible = 1;
			if (!anyVisible) c->occluded = 1;
		}
	}
	target tg;
	memset(&tg, 0, sizeof(tg));
	tg.color = r->color; tg.depth = r->depth; tg.width = r->width; tg.height = r->height;
	tg.packOrder = r->packOrder; tg.stats = stats;
	irect imageBound = {0, 0, r->width, r->height};
	row_interval *rows = NULL;
	int32_t capacity = 0;
	for (size_t i = 0; i < r->commands.count; i++) {
		const command *c = &r->commands.items[i];
		if (!c->occluded) execute_command(c, &r->cams[c->task], &tg, imageBound, imageBound, &rows, &capacity);
	}
	free(rows);
	if (stats) stats->fragments += tg.fragments;
	if (r->color) {
		if (debugWireframe) {
			for (size_t i = 0; i < r->commands.count; i++) {
				const command *c = &r->commands.items[i];
				if (c->occluded) continue;
				const projected *p = c->triangle.position;
				for (int e = 0; e < 3; e++) {
					const projected *a = &p[e], *b = &p[(e + 1) % 3];
					draw_line(r->color, r->width, r->height, (int32_t)(a->flat.x / 256), (int32_t)(a->flat.y / 256),
					          (int32_t)(b->flat.x / 256), (int32_t)(b->flat.y / 256), 0xFFFFFFFFu);
				}
			}
		}
		for (int32_t l = 0; l < r->debugCount; l++) {
			const debug_line *d = &r->debugLines[l];
			uint32_t packed = 0; /* image_saturateAndPack in the target's pack order */
			for (int ch = 0; ch < 4; ch++) packed |= ((d->color >> (ch * 8)) & 0xFFu) << (PACK_INDEX[r->packOrder][ch] * 8);
			draw_line(r->color, r->width, r->height, d->x1, d->y1, d->x2, d->y2, packed);
		}
		r->debugCount = 0;
	}
	r->commands.count = 0;
	return 0;
}

/* The grid as isBoxVisible reads it (for tests); returns whether an occluder was given this frame. */
int or_renderer_grid(const or_renderer *r, float *out, int32_t *gridWidth, int32_t *gridHeight) {
	*gridWidth = r->gridWidth;
	*gridHeight = r->gridHeight;
	if (!out) return r->occluded;
	for (int32_t y = 0; y < r->gridHeight; y++)
		for (int32_t x = 0; x < r->gridWidth; x++) out[(size_t)y * r->gridWidth + x] = grid_read(r, x, y);
	return r->occluded;
}

/* ---- dense models of the sprite engine (SDK/SpriteEngine/spriteAPI.cpp:236-262, 1143-1327) ---- */

int32_t or_dense_triangle_count(const int32_t *polygons, int32_t polygonCount) {
	int32_t n = 0;
	for (int32_t p = 0; p < polygonCount; p++) n += polygons[p * 4 + 3] < 0 ? 1 : 2;
	return n;
}

/* DenseModelImpl::DenseModelImpl (spriteAPI.cpp:1189-1240): smooth normals (each polygon's
 * normalized sum of its fan triangles' normals added to its points, then normalized per point),
 * colours times 255, one dense triangle per fan triangle of every polygon in order. */
void or_dense_model_create(const float *positions, int32_t pointCount, const int32_t *polygons, const float *colors,
                           int32_t polygonCount, or_dense_triangle *out) {
	v3 *normals = (v3 *)calloc((size_t)(pointCount > 0 ? pointCount : 1), sizeof(v3));
	for (int32_t p = 0; p < polygonCount; p++) {
		const int32_t *idx = polygons + p * 4;
		const int32_t corners = idx[3] < 0 ? 3 : 4;
		v3 sum = mk3(0.0f, 0.0f, 0.0f);
		const v3 a = mk3(positions[idx[0] * 3], positions[idx[0] * 3 + 1], positions[idx[0] * 3 + 2]);
		for (int32_t t = 0; t < corners - 2; t++) { /* getAverageNormal (spriteAPI.cpp:1160-1171) */
			const int32_t ib = idx[t + 1], ic = idx[t + 2];
			const v3 b = mk3(positions[ib * 3], positions[ib * 3 + 1], positions[ib * 3 + 2]);
			const v3 c = mk3(positions[ic * 3], positions[ic * 3 + 1], positions[ic * 3 + 2]);
			sum = add3(sum, normalize3(cross3(sub3(b, a), sub3(c, a))));
		}
		const v3 n = normalize3(sum);
		for (int32_t v = 0; v < corners; v++) normals[idx[v]] = add3(normals[idx[v]], n);
	}
	for (int32_t i = 0; i < pointCount; i++) normals[i] = normalize3(normals[i]);
	int32_t t = 0;
	for (int32_t p = 0; p < polygonCount; p++) {
		const int32_t *idx = polygons + p * 4;
		const int32_t corners = idx[3] < 0 ? 3 : 4;
		for (int32_t vb = 1; vb < corners - 1; vb++) {
			const int32_t vert[3] = {0, vb, vb + 1};
			or_dense_triangle *d = &out[t++];
			for (int32_t k = 0; k < 3; k++) {
				const float *col = colors + (p * 4 + vert[k]) * 4;
				const int32_t point = idx[vert[k]];
				d->color[k][0] = col[0] * 255.0f; d->color[k][1] = col[1] * 255.0f; d->color[k][2] = col[2] * 255.0f;
				d->pos[k][0] = positions[point * 3]; d->pos[k][1] = positions[point * 3 + 1]; d->pos[k][2] = positions[point * 3 + 2];
				d->normal[k][0] = normals[point].x; d->normal[k][1] = normals[point].y; d->normal[k][2] = normals[point].z;
			}
		}
	}
	free(normals);
}

static inline float dense_min3(float a, float b, float c) { const float m = a < b ? a : b; return m < c ? m : c; } /* base/noSimd.h:134-140 */
static inline float dense_max3(float a, float b, float c) { const float m = a > b ? a : b; return m > c ? m : c; }
/* (uint32_t)float of the reference's x86-64 build: a signed 64-bit truncation keeping the low 32 bits. */
static inline uint32_t dense_u32(float x) { return (uint32_t)(int64_t)x; }

/* renderDenseModel<HIGH_QUALITY> (spriteAPI.cpp:1244-1327) into height, diffuse and normal images
 * (strides in elements).  The pessimistic bounding-box test only skips models that draw nothing,
 * so it is left out. */
void or_dense_render(const or_dense_triangle *triangles, int32_t count, const or_ortho_view *view, float *height,
                     int32_t heightStride, uint32_t *diffuse, int32_t diffuseStride, uint32_t *normal, int32_t normalStride,
                     int32_t width, int32_t heightPx, float originX, float originY, const float modelToWorld[12],
                     int32_t highQuality) {
	/* combineModelToScreenTransform (spriteAPI.cpp:29-35) with Transform3D's product (Transform3D.h:56-58) */
	m3 tileToScreen;
	tileToScreen.x = mk3((float)view->pixelOffsetPerTileX[0], (float)view->pixelOffsetPerTileX[1], 0.0f);
	tileToScreen.y = mk3(0.0f, (float)(-view->yPixelsPerTile), 1.0f);
	tileToScreen.z = mk3((float)view->pixelOffsetPerTileZ[0], (float)view->pixelOffsetPerTileZ[1], 0.0f);
	m3 model;
	model.x = mk3(modelToWorld[3], modelToWorld[4], modelToWorld[5]);
	model.y = mk3(modelToWorld[6], modelToWorld[7], modelToWorld[8]);
	model.z = mk3(modelToWorld[9], modelToWorld[10], modelToWorld[11]);
	const v3 position = add3(m3_transform(&tileToScreen, mk3(modelToWorld[0], modelToWorld[1], modelToWorld[2])), mk3(originX, originY, 0.0f));
	const m3 toScreen = m3_mul(&model, &tileToScreen);
	m3 n, nt; /* transpose(normalToWorldSpace) (FMatrix3x3.h:109-120) */
	n.x = mk3(view->normalToWorld[0], view->normalToWorld[1], view->normalToWorld[2]);
	n.y = mk3(view->normalToWorld[3], view->normalToWorld[4], view->normalToWorld[5]);
	n.z = mk3(view->normalToWorld[6], view->normalToWorld[7], view->normalToWorld[8]);
	nt.x = mk3(n.x.x, n.y.x, n.z.x); nt.y = mk3(n.x.y, n.y.y, n.z.y); nt.z = mk3(n.x.z, n.y.z, n.z.z);
	const m3 toNormal = m3_mul(&model, &nt);
	for (int32_t t = 0; t < count; t++) {
		const or_dense_triangle *d = &triangles[t];
		v3 p[3], nn[3];
		for (int32_t k = 0; k < 3; k++) {
			p[k] = add3(m3_transform(&toScreen, mk3(d->pos[k][0], d->pos[k][1], d->pos[k][2])), position);
		}
		const v3 a = p[0], b = p[1], c = p[2];
		/* getBackCulledTriangleBound (spriteAPI.cpp:1143-1155), cut to the image (IRect.h:56-66) */
		if (((c.x - a.x) * (b.y - a.y)) + ((c.y - a.y) * (a.x - b.x)) >= 0.0f) continue;
		const int32_t left = (int32_t)dense_min3(a.x, b.x, c.x), top = (int32_t)dense_min3(a.y, b.y, c.y);
		const int32_t right = (int32_t)dense_max3(a.x, b.x, c.x) + 1, bottom = (int32_t)dense_max3(a.y, b.y, c.y) + 1;
		if (!(left < width && right > 0 && top < heightPx && bottom > 0)) continue;
		const int32_t x0 = left > 0 ? left : 0, y0 = top > 0 ? top : 0;
		const int32_t x1 = right < width ? right : width, y1 = bottom < heightPx ? bottom : heightPx;
		if (x1 <= x0 || y1 <= y0) continue;
		/* inverse(FMatrix2x2(B - A, C - A)) (FMatrix2x2.h:69-76) */
		const float mxx = b.x - a.x, mxy = b.y - a.y, myx = c.x - a.x, myy = c.y - a.y;
		const float invDet = 1.0f / (mxx * myy - mxy * myx);
		const float ixx = myy * invDet, ixy = -mxy * invDet, iyx = -myx * invDet, iyy = mxx * invDet;
		for (int32_t k = 0; k < 3; k++) nn[k] = m3_transform(&toNormal, mk3(d->normal[k][0], d->normal[k][1], d->normal[k][2]));
		for (int32_t y = y0; y < y1; y++) {
			for (int32_t x = x0; x < x1; x++) {
				const float ox = ((float)x + 0.5f) - a.x, oy = ((float)y + 0.5f) - a.y;
				const float wb = ox * ixx + oy * iyx, wc = ox * ixy + oy * iyy;
				const float wa = 1.0f - (wb + wc);
				if (!(wa >= -0.00001f && wb >= -0.00001f && wc >= -0.00001f)) continue;
				const float h = a.z * wa + b.z * wb + c.z * wc; /* interpolateUsingAffineWeight (ITriangle2D.h:58-61) */
				float *target = &height[(size_t)y * heightStride + x];
				if (!(h > *target)) continue;
				*target = h;
				float col[3], nv[3];
				for (int32_t ch = 0; ch < 3; ch++) col[ch] = d->color[0][ch] * wa + d->color[1][ch] * wb + d->color[2][ch] * wc;
				v3 nsum = mk3(nn[0].x * wa + nn[1].x * wb + nn[2].x * wc, nn[0].y * wa + nn[1].y * wb + nn[2].y * wc,
				              nn[0].z * wa + nn[1].z * wb + nn[2].z * wc);
				if (highQuality) nsum = normalize3(nsum);
				nv[0] = (nsum.x + 1.0f) * 127.5f; nv[1] = (nsum.y + 1.0f) * 127.5f; nv[2] = (nsum.z + 1.0f) * 127.5f;
				diffuse[(size_t)y * diffuseStride + x] = dense_u32(col[0]) | (dense_u32(col[1]) << 8) | (dense_u32(col[2]) << 16) | (255u << 24);
				normal[(size_t)y * normalStride + x] = dense_u32(nv[0]) | (dense_u32(nv[1]) << 8) | (dense_u32(nv[2]) << 16) | (255u << 24);
			}
		}
	}
}
