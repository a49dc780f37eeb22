// Vertex projection, culling, clipping and triangle setup of the DFPSR triangle path,
// shared by the kernels and the host.  Float operations follow the reference's
// order one by one (no contraction), so corners and projections are bit-identical.
#ifndef DSRG_GEOMETRY_H
#define DSRG_GEOMETRY_H

#include "dsrg_exact.h"
#include "dsrg_types.h"

namespace dsrg {

struct Vec3 { float x, y, z; };

DSRG_HD Vec3 vec3(float x, float y, float z) { Vec3 v; v.x = x; v.y = y; v.z = z; return v; }
DSRG_HD float dot3(const Vec3 &a, float nx, float ny, float nz) { // math/FVector.h:74-76
	return fadd(fadd(fmul(a.x, nx), fmul(a.y, ny)), fmul(a.z, nz));
}

// Transform3D::transformPoint (math/Transform3D.h:39-41, FMatrix3x3.h:55-61); m = position, x, y, z axes.
DSRG_HD Vec3 transform_point(const float *m, const Vec3 &p) {
	float x = fadd(fadd(fmul(p.x, m[3]), fmul(p.y, m[6])), fmul(p.z, m[9]));
	float y = fadd(fadd(fmul(p.x, m[4]), fmul(p.y, m[7])), fmul(p.z, m[10]));
	float z = fadd(fadd(fmul(p.x, m[5]), fmul(p.y, m[8])), fmul(p.z, m[11]));
	return vec3(fadd(x, m[0]), fadd(y, m[1]), fadd(z, m[2]));
}

// Camera::worldToCamera (implementation/render/Camera.h:157-159; math/Transform3D.h:49-51, FMatrix3x3.h:66-72).
DSRG_HD Vec3 world_to_camera(const CameraData &c, const Vec3 &p) {
	Vec3 d = vec3(p.x - c.position[0], p.y - c.position[1], p.z - c.position[2]);
	return vec3(fadd(fadd(fmul(d.x, c.xAxis[0]), fmul(d.y, c.xAxis[1])), fmul(d.z, c.xAxis[2])),
	            fadd(fadd(fmul(d.x, c.yAxis[0]), fmul(d.y, c.yAxis[1])), fmul(d.z, c.yAxis[2])),
	            fadd(fadd(fmul(d.x, c.zAxis[0]), fmul(d.y, c.zAxis[1])), fmul(d.z, c.zAxis[2])));
}

struct Projected {
	Vec3 cs;
	float isx, isy;
	int64_t flatx, flaty;
};

// Camera::cameraToScreen (implementation/render/Camera.h:160-187).
DSRG_HD Projected camera_to_screen(const CameraData &c, const Vec3 &cs) {
	Projected p;
	p.cs = cs;
	if (c.perspective) {
		float invDepth = (cs.z > 0.0f) ? frcp(cs.z) : 0.0f;
		float centerShear = fmul(cs.z, 0.5f);
		float preX = fmul(fadd(fmul(cs.x, c.invWidthSlope), centerShear), c.imageWidth);
		float preY = fmul(fadd(fmul(-cs.y, c.invHeightSlope), centerShear), c.imageHeight);
		p.isx = fmul(preX, invDepth);
		p.isy = fmul(preY, invDepth);
	} else {
		p.isx = fmul(fadd(fmul(cs.x, c.invWidthSlope), 0.5f), c.imageWidth);
		p.isy = fmul(fadd(fmul(-cs.y, c.invHeightSlope), 0.5f), c.imageHeight);
	}
	p.flatx = (int64_t)fmul(p.isx, 256.0f);
	p.flaty = (int64_t)fmul(p.isy, 256.0f);
	return p;
}

DSRG_HD bool plane_inside(const Plane &pl, const Vec3 &p) { // math/FPlane3D.h:38-46
	return fadd(dot3(p, pl.nx, pl.ny, pl.nz), -pl.offset) <= 0.0f;
}

// getTriangleVisibility (implementation/render/renderCore.cpp:172-198): 0 hidden, 1 full, 2 partial.
DSRG_HD int triangle_visibility(const CameraData &c, const Vec3 &a, const Vec3 &b, const Vec3 &d, bool clipFrustum) {
	const int count = clipFrustum ? c.clipCount : c.cullCount;
	const Plane *planes = clipFrustum ? c.clip : c.cull;
	bool anyOutside = false;
	for (int s = 0; s < count; s++) {
		bool oa = !plane_inside(planes[s], a), ob = !plane_inside(planes[s], b), od = !plane_inside(planes[s], d);
		if (oa && ob && od) return 0;
		anyOutside = anyOutside || oa || ob || od;
	}
	return anyOutside ? 2 : 1;
}

// ITriangle2D::isFrontfacing (implementation/render/ITriangle2D.cpp:55-60).
DSRG_HD bool is_frontfacing(const int64_t *fx, const int64_t *fy) {
	return ((fx[2] - fx[0]) * (fy[1] - fy[0])) + ((fy[2] - fy[0]) * (fx[0] - fx[1])) < 0;
}

// getTriangleBound (ITriangle2D.cpp:31-43) as exclusive bounds left, top, right, bottom.
DSRG_HD void triangle_bound(const int64_t *fx, const int64_t *fy, int32_t *bound) {
	int32_t rx[3], ry[3];
	for (int i = 0; i < 3; i++) {
		rx[i] = (int32_t)((fx[i] + 128) / 256);
		ry[i] = (int32_t)((fy[i] + 128) / 256);
	}
	int32_t l = rx[0], t = ry[0], r = rx[0], b = ry[0];
	for (int i = 1; i < 3; i++) {
		l = rx[i] < l ? rx[i] : l; t = ry[i] < t ? ry[i] : t;
		r = rx[i] > r ? rx[i] : r; b = ry[i] > b ? ry[i] : b;
	}
	bound[0] = l - 1; bound[1] = t - 1; bound[2] = r + 1; bound[3] = b + 1;
}

// ITriangle2D::getProjection (implementation/render/ITriangle2D.cpp:182-300).
// is: 3 x (x, y); csz: camera-space depth of the corners; out: start, dx, dy (3 floats each).
DSRG_HD void triangle_projection(const float *isx, const float *isy, const float *csz, const float *subB,
                                 const float *subC, bool perspective, float *start, float *dx, float *dy) {
	float offsetX[3], offsetY[3], weightMultiplier[3], normalX[3], normalY[3], targetWeight[3];
	for (int i = 0; i < 3; i++) {
		int j = (i + 1) % 3;
		offsetX[i] = isy[j] - isy[i];
		offsetY[i] = isx[i] - isx[j];
	}
	for (int i = 0; i < 3; i++) {
		int o = (i + 2) % 3;
		float other = fadd(fmul(isx[o] - isx[i], offsetX[i]), fmul(isy[o] - isy[i], offsetY[i]));
		weightMultiplier[o] = (other == 0.0f) ? 0.0f : frcp(other);
	}
	for (int i = 0; i < 3; i++) {
		normalX[i] = fmul(offsetX[i], weightMultiplier[i]);
		normalY[i] = fmul(offsetY[i], weightMultiplier[i]);
	}
	for (int i = 0; i < 3; i++) {
		int o = (i + 2) % 3;
		targetWeight[o] = fadd(fmul(isx[i], -normalX[i]), fmul(isy[i], -normalY[i]));
	}
	const float awdx[3] = {normalX[1], normalX[2], normalX[0]};
	const float awdy[3] = {normalY[1], normalY[2], normalY[0]};
	if (!perspective) {
		const float *W = csz;
		start[0] = fadd(fadd(fmul(W[0], targetWeight[0]), fmul(W[1], targetWeight[1])), fmul(W[2], targetWeight[2]));
		start[1] = fadd(fadd(fmul(targetWeight[0], subB[0]), fmul(targetWeight[1], subB[1])), fmul(targetWeight[2], subB[2]));
		start[2] = fadd(fadd(fmul(targetWeight[0], subC[0]), fmul(targetWeight[1], subC[1])), fmul(targetWeight[2], subC[2]));
		dx[0] = fadd(fadd(fmul(W[0], awdx[0]), fmul(W[1], awdx[1])), fmul(W[2], awdx[2]));
		dx[1] = fadd(fadd(fmul(awdx[0], subB[0]), fmul(awdx[1], subB[1])), fmul(awdx[2], subB[2]));
		dx[2] = fadd(fadd(fmul(awdx[0], subC[0]), fmul(awdx[1], subC[1])), fmul(awdx[2], subC[2]));
		dy[0] = fadd(fadd(fmul(W[0], awdy[0]), fmul(W[1], awdy[1])), fmul(W[2], awdy[2]));
		dy[1] = fadd(fadd(fmul(awdy[0], subB[0]), fmul(awdy[1], subB[1])), fmul(awdy[2], subB[2]));
		dy[2] = fadd(fadd(fmul(awdy[0], subC[0]), fmul(awdy[1], subC[1])), fmul(awdy[2], subC[2]));
	} else {
		const float IW[3] = {frcp(csz[0]), frcp(csz[1]), frcp(csz[2])};
		start[0] = fadd(fadd(fmul(IW[0], targetWeight[0]), fmul(IW[1], targetWeight[1])), fmul(IW[2], targetWeight[2]));
		start[1] = fadd(fadd(fmul(fmul(IW[0], targetWeight[0]), subB[0]), fmul(fmul(IW[1], targetWeight[1]), subB[1])),
		                fmul(fmul(IW[2], targetWeight[2]), subB[2]));
		start[2] = fadd(fadd(fmul(fmul(IW[0], targetWeight[0]), subC[0]), fmul(fmul(IW[1], targetWeight[1]), subC[1])),
		                fmul(fmul(IW[2], targetWeight[2]), subC[2]));
		dx[0] = fadd(fadd(fmul(IW[0], awdx[0]), fmul(IW[1], awdx[1])), fmul(IW[2], awdx[2]));
		dx[1] = fadd(fadd(fmul(fmul(IW[0], awdx[0]), subB[0]), fmul(fmul(IW[1], awdx[1]), subB[1])), fmul(fmul(IW[2], awdx[2]), subB[2]));
		dx[2] = fadd(fadd(fmul(fmul(IW[0], awdx[0]), subC[0]), fmul(fmul(IW[1], awdx[1]), subC[1])), fmul(fmul(IW[2], awdx[2]), subC[2]));
		dy[0] = fadd(fadd(fmul(IW[0], awdy[0]), fmul(IW[1], awdy[1])), fmul(IW[2], awdy[2]));
		dy[1] = fadd(fadd(fmul(fmul(IW[0], awdy[0]), subB[0]), fmul(fmul(IW[1], awdy[1]), subB[1])), fmul(fmul(IW[2], awdy[2]), subB[2]));
		dy[2] = fadd(fadd(fmul(fmul(IW[0], awdy[0]), subC[0]), fmul(fmul(IW[1], awdy[1]), subC[1])), fmul(fmul(IW[2], awdy[2]), subC[2]));
	}
}

// Sub-vertex of a clipped triangle (implementation/render/renderCore.cpp:33-47).
struct SubVertex {
	Vec3 cs;
	float subB, subC;
	int32_t state;
	float value;
};

DSRG_HD SubVertex sub_lerp(const SubVertex &a, const SubVertex &b, float ratio) {
	SubVertex r;
	float inv = 1.0f - ratio;
	r.cs = vec3(fadd(fmul(a.cs.x, inv), fmul(b.cs.x, ratio)), fadd(fmul(a.cs.y, inv), fmul(b.cs.y, ratio)),
	            fadd(fmul(a.cs.z, inv), fmul(b.cs.z, ratio)));
	r.subB = fadd(fmul(a.subB, inv), fmul(b.subB, ratio));
	r.subC = fadd(fmul(a.subC, inv), fmul(b.subC, ratio));
	r.state = 0;
	r.value = 0.0f;
	return r;
}

DSRG_HD float inverse_lerp(float a, float b, float value) { // renderCore.cpp:52-59
	float c = b - a;
	return (c == 0.0f) ? 0.5f : fdiv(value - a, c);
}

static const int MAX_CLIP_POINTS = 9;

// ClippedTriangle (renderCore.cpp:61-170): a convex polygon of at most 9 corners.
struct ClippedPolygon {
	int32_t count;
	SubVertex v[MAX_CLIP_POINTS];

	DSRG_HD void remove(int index) {
		if (count > 0 && count <= MAX_CLIP_POINTS) {
			for (int i = index; i < count - 1; i++) v[i] = v[i + 1];
			count--;
		}
	}
	DSRG_HD void insert(int index, const SubVertex &nv) {
		if (count < MAX_CLIP_POINTS) {
			for (int i = count - 1; i >= index; i--) v[i + 1] = v[i];
			v[index] = nv;
			count++;
		}
	}
	// ClippedTriangle::clip (renderCore.cpp:104-169).
	DSRG_HD void clip(const Plane &p) {
		if (!(count >= 3 && count < MAX_CLIP_POINTS)) return;
		int outsideCount = 0, lastOutside = 0;
		for (int i = 0; i < count; i++) {
			float distance = fadd(dot3(v[i].cs, p.nx, p.ny, p.nz), -p.offset);
			v[i].value = distance;
			if (distance > 0.0f) { outsideCount++; lastOutside = i; v[i].state = 1; } else { v[i].state = 0; }
		}
		if (outsideCount == 0) return;
		if (outsideCount >= count) {
			count = 0;
		} else if (outsideCount == 1) {
			int cur = lastOutside;
			int prev = (lastOutside - 1 + count) % count;
			int next = (lastOutside + 1) % count;
			float r0 = inverse_lerp(v[prev].value, v[cur].value, 0.0f);
			float r1 = inverse_lerp(v[cur].value, v[next].value, 0.0f);
			SubVertex cutStart = sub_lerp(v[prev], v[cur], r0);
			SubVertex cutEnd = sub_lerp(v[cur], v[next], r1);
			v[lastOutside] = cutStart;
			insert(next, cutEnd);
		} else {
			for (int cur = 0; cur < count; cur++) {
				int prev = (cur - 1 + count) % count;
				int next = (cur + 1) % count;
				if (v[cur].state == 1) {
					if (v[prev].state == 0) {
						float r = inverse_lerp(v[prev].value, v[cur].value, 0.0f);
						v[cur] = sub_lerp(v[prev], v[cur], r);
						v[cur].state = 2;
					} else if (v[next].state == 0) {
						float r = inverse_lerp(v[cur].value, v[next].value, 0.0f);
						v[cur] = sub_lerp(v[cur], v[next], r);
						v[cur].state = 2;
					}
				}
			}
			if (outsideCount > 2) {
				for (int i = count - 1; i >= 0; i--)
					if (v[i].state == 1) remove(i);
			}
		}
	}
};

} // namespace dsrg

#endif
