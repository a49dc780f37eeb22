// The renderer's occlusion grid (RendererImpl, api/rendererAPI.cpp:141-477), shared by the
// kernels and the host.  One float per 16x16-pixel cell holds the largest camera-space depth at
// which something in the cell may still be visible (infinity while nothing occludes it).
// Occluders lower cells that their convex hull covers completely; a draw command whose nearest
// corner lies behind every cell of its bound is not drawn.  All tests are the reference's own
// integer hull tests on sub-pixel coordinates and its float (and one double) comparisons.
#ifndef DSRG_OCCLUSION_H
#define DSRG_OCCLUSION_H

#include "dsrg_exact.h"

namespace dsrg {

const int32_t OCCLUSION_CELL = 16;

struct CellRect { int32_t left, top, right, bottom; };

// getOuterCellBound (rendererAPI.cpp:168-179) of an exclusive pixel bound.
DSRG_HD CellRect outer_cell_bound(int32_t left, int32_t top, int32_t right, int32_t bottom, int32_t gridWidth, int32_t gridHeight) {
	CellRect c;
	c.left = left / OCCLUSION_CELL;
	c.right = right / OCCLUSION_CELL + 1;
	c.top = top / OCCLUSION_CELL;
	c.bottom = bottom / OCCLUSION_CELL + 1;
	if (c.left < 0) c.left = 0;
	if (c.top < 0) c.top = 0;
	if (c.right > gridWidth) c.right = gridWidth;
	if (c.bottom > gridHeight) c.bottom = gridHeight;
	return c;
}

// pointInsideOfHull with pointInsideOfEdge (rendererAPI.cpp:100-121): the hull's corners in order,
// the point inside or on every edge.
DSRG_HD bool point_inside_hull(const int64_t *hx, const int64_t *hy, int32_t count, int64_t px, int64_t py) {
	for (int32_t c = 0; c < count; c++) {
		const int32_t nc = (c + 1 == count) ? 0 : c + 1;
		const int64_t ex = hy[nc] - hy[c], ey = hx[c] - hx[nc];
		if (!(ex * (px - hx[c]) + ey * (py - hy[c]) <= 0)) return false;
	}
	return true;
}

// rectangleInsideOfHull (rendererAPI.cpp:124-130) for the cell's sub-pixel rectangle.
DSRG_HD bool cell_inside_hull(const int64_t *hx, const int64_t *hy, int32_t count, int32_t cellX, int32_t cellY) {
	const int64_t left = (int64_t)(cellX * OCCLUSION_CELL * 256), top = (int64_t)(cellY * OCCLUSION_CELL * 256);
	const int64_t right = left + OCCLUSION_CELL * 256, bottom = top + OCCLUSION_CELL * 256;
	return point_inside_hull(hx, hy, count, left, top) && point_inside_hull(hx, hy, count, right, top) &&
	       point_inside_hull(hx, hy, count, left, bottom) && point_inside_hull(hx, hy, count, right, bottom);
}

// completeOcclusion's test of one draw command (rendererAPI.cpp:193-214): visible when some cell
// of its outer cell bound is not nearer than its nearest corner by more than 0.001 (compared in
// double, as the reference's double literal makes it).
DSRG_HD bool command_survives(const float *grid, int32_t gridWidth, int32_t gridHeight, int32_t gridStride, const int32_t *bound,
                              float nearest) {
	const CellRect cells = outer_cell_bound(bound[0], bound[1], bound[2], bound[3], gridWidth, gridHeight);
	for (int32_t cy = cells.top; cy < cells.bottom; cy++)
		for (int32_t cx = cells.left; cx < cells.right; cx++)
			if ((double)nearest < (double)grid[(size_t)cy * gridStride + cx] + 0.001) return true;
	return false;
}

// replaceWithSmaller over the three corners, in the reference's order.
DSRG_HD float nearest_corner(float z0, float z1, float z2) {
	float z = z0;
	if (z1 < z) z = z1;
	if (z2 < z) z = z2;
	return z;
}

} // namespace dsrg

#endif
