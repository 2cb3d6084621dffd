/*
 * cpg_narrow.cuh -- per-pair narrow phase (src/cpCollision.c) on the device.
 *
 * One thread handles one candidate pair: the shapes are ordered by kind
 * (cpCollision.c:701-726) and dispatched to the circle/segment/polygon
 * routine.  GJK (:416-472) and EPA (:270-343) run as bounded loops (the
 * reference's recursion caps of 30 iterations each), with the EPA hull in
 * registers/local memory.  Contact points, normals and feature hashes are
 * produced with the reference's arithmetic, in the same order.
 */
#pragma once
#ifdef __CUDACC__
#include <math_constants.h>
#endif
#include "cpg_device.h"
#include "cpg_math.cuh"

/* A shape's world-space data gathered for the narrow phase. */
struct ShapeView {
	int kind;
	double r;
	V2 p0, p1, n;            /* circle: tc | segment: ta, tb, tn */
	V2 atan, btan;           /* segment tangents (body space) */
	V2 rot;                  /* body rotation (transform a, b) */
	BB bb;
	unsigned long long hashid;
	int count;               /* polygon vertex count */
	const double *vx, *vy, *nx, *ny;   /* polygon world planes */
};

struct NarrowCtx {
	const cpgSet *s;
	int shapeBase, bodyBase, vertBase;
};

static __device__ ShapeView load_shape(const NarrowCtx &c, int shape)
{
	const cpgSet *s = c.s;
	int g = c.shapeBase + shape;
	ShapeView v;
	v.kind = s->skind[g];
	v.r = s->sr[g];
	v.p0 = v2(s->w0x[g], s->w0y[g]);
	v.p1 = v2(s->w1x[g], s->w1y[g]);
	v.n = v2(s->wnx[g], s->wny[g]);
	v.atan = v2(s->atx[g], s->aty[g]);
	v.btan = v2(s->btx[g], s->bty[g]);
	int body = c.bodyBase + s->sbody[g];
	v.rot = v2(s->ta[body], s->tb[body]);
	v.bb = bbnew(s->bbl[g], s->bbb[g], s->bbr[g], s->bbt[g]);
	v.hashid = s->shash[g];
	int voff = c.vertBase + s->svoff[g];
	v.count = s->svcount[g];
	v.vx = s->gvx + voff; v.vy = s->gvy + voff;
	v.nx = s->gnx + voff; v.ny = s->gny + voff;
	return v;
}

struct NInfo {
	V2 n;
	int count;
	unsigned id;
	V2 p1[2], p2[2];
	unsigned long long hash[2];
};

__device__ __forceinline__ void push_contact(NInfo &info, V2 p1, V2 p2, unsigned long long hash)
{
	if(info.count < 2){
		info.p1[info.count] = p1;
		info.p2[info.count] = p2;
		info.hash[info.count] = hash;
	}
	info.count++;
}

/* cpRobust.c:5-13 */
__device__ __forceinline__ bool check_point_greater(V2 a, V2 b, V2 c)
{
	return (b.y - a.y)*(a.x + b.x - 2*c.x) > (b.x - a.x)*(a.y + b.y - 2*c.y);
}

__device__ __forceinline__ bool check_axis(V2 v0, V2 v1, V2 p, V2 n)
{
	return vdot(p, n) <= dmax(vdot(v0, n), vdot(v1, n));
}

struct SPt { V2 p; unsigned index; };
struct MPt { V2 a, b, ab; unsigned id; };

/* cpCollision.c:62-76 */
static __device__ int poly_support_index(const ShapeView &s, V2 n)
{
	double max = -CUDART_INF;
	int index = 0;
	for(int i = 0; i < s.count; i++){
		double d = vdot(v2(s.vx[i], s.vy[i]), n);
		if(d > max){ max = d; index = i; }
	}
	return index;
}

/* cpCollision.c:86-110 */
static __device__ SPt support_point(const ShapeView &s, V2 n)
{
	SPt sp;
	if(s.kind == CPG_CIRCLE){
		sp.p = s.p0; sp.index = 0;
	} else if(s.kind == CPG_SEGMENT){
		if(vdot(s.p0, n) > vdot(s.p1, n)){ sp.p = s.p0; sp.index = 0; }
		else { sp.p = s.p1; sp.index = 1; }
	} else {
		int i = poly_support_index(s, n);
		sp.p = v2(s.vx[i], s.vy[i]); sp.index = (unsigned)i;
	}
	return sp;
}

__device__ __forceinline__ MPt minkowski(SPt a, SPt b)
{
	MPt m; m.a = a.p; m.b = b.p; m.ab = vsub(b.p, a.p);
	m.id = (a.index & 0xFF) << 8 | (b.index & 0xFF);
	return m;
}

__device__ __forceinline__ MPt support(const ShapeView &s1, const ShapeView &s2, V2 n)
{
	return minkowski(support_point(s1, vneg(n)), support_point(s2, n));
}

struct EdgePt { V2 p; unsigned long long hash; };
struct Edge { EdgePt a, b; double r; V2 n; };

/* cpCollision.c:163-182 */
static __device__ Edge support_edge_poly(const ShapeView &poly, V2 n)
{
	int count = poly.count;
	int i1 = poly_support_index(poly, n);
	int i0 = (i1 - 1 + count)%count;
	int i2 = (i1 + 1)%count;
	Edge e;
	V2 n1 = v2(poly.nx[i1], poly.ny[i1]), n2 = v2(poly.nx[i2], poly.ny[i2]);
	if(vdot(n, n1) > vdot(n, n2)){
		e.a.p = v2(poly.vx[i0], poly.vy[i0]); e.a.hash = hash_pair(poly.hashid, (unsigned long long)i0);
		e.b.p = v2(poly.vx[i1], poly.vy[i1]); e.b.hash = hash_pair(poly.hashid, (unsigned long long)i1);
		e.r = poly.r; e.n = n1;
	} else {
		e.a.p = v2(poly.vx[i1], poly.vy[i1]); e.a.hash = hash_pair(poly.hashid, (unsigned long long)i1);
		e.b.p = v2(poly.vx[i2], poly.vy[i2]); e.b.hash = hash_pair(poly.hashid, (unsigned long long)i2);
		e.r = poly.r; e.n = n2;
	}
	return e;
}

/* cpCollision.c:184-195 */
static __device__ Edge support_edge_segment(const ShapeView &seg, V2 n)
{
	Edge e;
	if(vdot(seg.n, n) > 0.0){
		e.a.p = seg.p0; e.a.hash = hash_pair(seg.hashid, 0ull);
		e.b.p = seg.p1; e.b.hash = hash_pair(seg.hashid, 1ull);
		e.r = seg.r; e.n = seg.n;
	} else {
		e.a.p = seg.p1; e.a.hash = hash_pair(seg.hashid, 1ull);
		e.b.p = seg.p0; e.b.hash = hash_pair(seg.hashid, 0ull);
		e.r = seg.r; e.n = vneg(seg.n);
	}
	return e;
}

/* cpCollision.c:199-212 */
__device__ __forceinline__ double closest_t(V2 a, V2 b)
{
	V2 delta = vsub(b, a);
	return -dclamp(vdot(delta, vadd(a, b))/(vlensq(delta) + DBL_MIN), -1.0, 1.0);
}

__device__ __forceinline__ V2 lerp_t(V2 a, V2 b, double t)
{
	double ht = 0.5*t;
	return vadd(vmul(a, 0.5 - ht), vmul(b, 0.5 + ht));
}

struct CPts { V2 a, b, n; double d; unsigned id; };

/* cpCollision.c:227-258 */
static __device__ CPts closest_points(const MPt &v0, const MPt &v1)
{
	double t = closest_t(v0.ab, v1.ab);
	V2 p = lerp_t(v0.ab, v1.ab, t);
	CPts r;
	r.a = lerp_t(v0.a, v1.a, t);
	r.b = lerp_t(v0.b, v1.b, t);
	r.id = (v0.id & 0xFFFF) << 16 | (v1.id & 0xFFFF);
	V2 delta = vsub(v1.ab, v0.ab);
	V2 n = vnormalize(vrperp(delta));
	double d = vdot(n, p);
	if(d <= 0.0 || (-1.0 < t && t < 1.0)){
		r.n = n; r.d = d;
	} else {
		double d2 = vlen(p);
		r.n = vmul(p, 1.0/(d2 + DBL_MIN));
		r.d = d2;
	}
	return r;
}

__device__ __forceinline__ double closest_dist(V2 v0, V2 v1)
{
	return vlensq(lerp_t(v0, v1, closest_t(v0, v1)));
}

#define CPG_EPA_MAX 30
#define CPG_GJK_MAX 30

/* EPA as a bounded loop (cpCollision.c:270-343). */
static __device__ CPts epa(const ShapeView &s1, const ShapeView &s2, MPt v0, MPt v1, MPt v2)
{
	MPt hull[CPG_EPA_MAX + 4], hull2[CPG_EPA_MAX + 4];
	int count = 3;
	hull[0] = v0; hull[1] = v1; hull[2] = v2;
	for(int iteration = 1;; iteration++){
		int mini = 0;
		double minDist = CUDART_INF;
		for(int j = 0, i = count - 1; j < count; i = j, j++){
			double d = closest_dist(hull[i].ab, hull[j].ab);
			if(d < minDist){ minDist = d; mini = i; }
		}
		MPt e0 = hull[mini];
		MPt e1 = hull[(mini + 1)%count];
		MPt p = support(s1, s2, vperp(vsub(e1.ab, e0.ab)));
		bool duplicate = (p.id == e0.id || p.id == e1.id);
		if(!duplicate && check_point_greater(e0.ab, e1.ab, p.ab) && iteration < CPG_EPA_MAX){
			int count2 = 1;
			hull2[0] = p;
			for(int i = 0; i < count; i++){
				int index = (mini + 1 + i)%count;
				V2 h0 = hull2[count2 - 1].ab;
				V2 h1 = hull[index].ab;
				V2 h2 = (i + 1 < count ? hull[(index + 1)%count] : p).ab;
				if(check_point_greater(h0, h2, h1)){
					hull2[count2] = hull[index];
					count2++;
				}
			}
			for(int i = 0; i < count2; i++) hull[i] = hull2[i];
			count = count2;
		} else {
			return closest_points(e0, e1);
		}
	}
}

/* GJK as a bounded loop (cpCollision.c:348-392). */
static __device__ CPts gjk_loop(const ShapeView &s1, const ShapeView &s2, MPt v0, MPt v1)
{
	int iteration = 1;
	for(int guard = 0; guard < 4*CPG_GJK_MAX + 8; guard++){
		if(iteration > CPG_GJK_MAX) return closest_points(v0, v1);
		if(check_point_greater(v1.ab, v0.ab, v2(0.0, 0.0))){
			MPt t = v0; v0 = v1; v1 = t;
			continue;
		}
		double t = closest_t(v0.ab, v1.ab);
		V2 n = (-1.0 < t && t < 1.0 ? vperp(vsub(v1.ab, v0.ab)) : vneg(lerp_t(v0.ab, v1.ab, t)));
		MPt p = support(s1, s2, n);
		if(check_point_greater(p.ab, v0.ab, v2(0.0, 0.0)) && check_point_greater(v1.ab, p.ab, v2(0.0, 0.0))){
			return epa(s1, s2, v0, p, v1);
		}
		if(check_axis(v0.ab, v1.ab, p.ab, n)) return closest_points(v0, v1);
		if(closest_dist(v0.ab, p.ab) < closest_dist(p.ab, v1.ab)) v1 = p; else v0 = p;
		iteration++;
	}
	return closest_points(v0, v1);
}

/* cpCollision.c:395-415 */
static __device__ SPt shape_point(const ShapeView &s, int i)
{
	SPt sp;
	if(s.kind == CPG_CIRCLE){ sp.p = s.p0; sp.index = 0; }
	else if(s.kind == CPG_SEGMENT){ sp.p = (i == 0 ? s.p0 : s.p1); sp.index = (unsigned)i; }
	else {
		int index = (i < s.count ? i : 0);
		sp.p = v2(s.vx[index], s.vy[index]); sp.index = (unsigned)index;
	}
	return sp;
}

/* cpCollision.c:416-472 */
static __device__ CPts gjk(const ShapeView &s1, const ShapeView &s2, unsigned &id)
{
	MPt v0, v1;
	if(id){
		v0 = minkowski(shape_point(s1, (id >> 24) & 0xFF), shape_point(s2, (id >> 16) & 0xFF));
		v1 = minkowski(shape_point(s1, (id >> 8) & 0xFF), shape_point(s2, id & 0xFF));
	} else {
		V2 axis = vperp(vsub(bbcenter(s1.bb), bbcenter(s2.bb)));
		v0 = support(s1, s2, axis);
		v1 = support(s1, s2, vneg(axis));
	}
	CPts pts = gjk_loop(s1, s2, v0, v1);
	id = pts.id;
	return pts;
}

/* cpCollision.c:477-518 */
static __device__ void contact_points(const Edge &e1, const Edge &e2, const CPts &pts, NInfo &info)
{
	double mindist = e1.r + e2.r;
	if(pts.d <= mindist){
		V2 n = info.n = pts.n;
		double d_e1_a = vcross(e1.a.p, n);
		double d_e1_b = vcross(e1.b.p, n);
		double d_e2_a = vcross(e2.a.p, n);
		double d_e2_b = vcross(e2.b.p, n);
		double e1_denom = 1.0/(d_e1_b - d_e1_a + DBL_MIN);
		double e2_denom = 1.0/(d_e2_b - d_e2_a + DBL_MIN);
		{
			V2 p1 = vadd(vmul(n,  e1.r), vlerp(e1.a.p, e1.b.p, dclamp01((d_e2_b - d_e1_a)*e1_denom)));
			V2 p2 = vadd(vmul(n, -e2.r), vlerp(e2.a.p, e2.b.p, dclamp01((d_e1_a - d_e2_a)*e2_denom)));
			double dist = vdot(vsub(p2, p1), n);
			if(dist <= 0.0) push_contact(info, p1, p2, hash_pair(e1.a.hash, e2.b.hash));
		}{
			V2 p1 = vadd(vmul(n,  e1.r), vlerp(e1.a.p, e1.b.p, dclamp01((d_e2_a - d_e1_a)*e1_denom)));
			V2 p2 = vadd(vmul(n, -e2.r), vlerp(e2.a.p, e2.b.p, dclamp01((d_e1_b - d_e2_a)*e2_denom)));
			double dist = vdot(vsub(p2, p1), n);
			if(dist <= 0.0) push_contact(info, p1, p2, hash_pair(e1.b.hash, e2.a.hash));
		}
	}
}

/* cpCollision.c:525-537 */
static __device__ void circle_circle(const ShapeView &c1, const ShapeView &c2, NInfo &info)
{
	double mindist = c1.r + c2.r;
	V2 delta = vsub(c2.p0, c1.p0);
	double distsq = vlensq(delta);
	if(distsq < mindist*mindist){
		double dist = sqrt(distsq);
		V2 n = info.n = (dist ? vmul(delta, 1.0/dist) : v2(1.0, 0.0));
		push_contact(info, vadd(c1.p0, vmul(n, c1.r)), vadd(c2.p0, vmul(n, -c2.r)), 0ull);
	}
}

/* cpCollision.c:539-569 */
static __device__ void circle_segment(const ShapeView &circle, const ShapeView &seg, NInfo &info)
{
	V2 seg_a = seg.p0, seg_b = seg.p1, center = circle.p0;
	V2 seg_delta = vsub(seg_b, seg_a);
	double ct = dclamp01(vdot(seg_delta, vsub(center, seg_a))/vlensq(seg_delta));
	V2 closest = vadd(seg_a, vmul(seg_delta, ct));
	double mindist = circle.r + seg.r;
	V2 delta = vsub(closest, center);
	double distsq = vlensq(delta);
	if(distsq < mindist*mindist){
		double dist = sqrt(distsq);
		V2 n = info.n = (dist ? vmul(delta, 1.0/dist) : seg.n);
		V2 rot = seg.rot;
		if((ct != 0.0 || vdot(n, vrotate(seg.atan, rot)) >= 0.0) &&
		   (ct != 1.0 || vdot(n, vrotate(seg.btan, rot)) >= 0.0)){
			push_contact(info, vadd(center, vmul(n, circle.r)), vadd(closest, vmul(n, -seg.r)), 0ull);
		}
	}
}

/* cpCollision.c:571-604 */
static __device__ void segment_segment(const ShapeView &s1, const ShapeView &s2, NInfo &info)
{
	CPts pts = gjk(s1, s2, info.id);
	V2 n = pts.n;
	V2 rot1 = s1.rot, rot2 = s2.rot;
	if(pts.d <= (s1.r + s2.r) && (
		(!veql(pts.a, s1.p0) || vdot(n, vrotate(s1.atan, rot1)) <= 0.0) &&
		(!veql(pts.a, s1.p1) || vdot(n, vrotate(s1.btan, rot1)) <= 0.0) &&
		(!veql(pts.b, s2.p0) || vdot(n, vrotate(s2.atan, rot2)) >= 0.0) &&
		(!veql(pts.b, s2.p1) || vdot(n, vrotate(s2.btan, rot2)) >= 0.0))){
		contact_points(support_edge_segment(s1, n), support_edge_segment(s2, vneg(n)), pts, info);
	}
}

/* cpCollision.c:606-627 */
static __device__ void poly_poly(const ShapeView &p1, const ShapeView &p2, NInfo &info)
{
	CPts pts = gjk(p1, p2, info.id);
	if(pts.d - p1.r - p2.r <= 0.0){
		contact_points(support_edge_poly(p1, pts.n), support_edge_poly(p2, vneg(pts.n)), pts, info);
	}
}

/* cpCollision.c:629-659 */
static __device__ void segment_poly(const ShapeView &seg, const ShapeView &poly, NInfo &info)
{
	CPts pts = gjk(seg, poly, info.id);
	V2 n = pts.n;
	V2 rot = seg.rot;
	if(pts.d - seg.r - poly.r <= 0.0 && (
		(!veql(pts.a, seg.p0) || vdot(n, vrotate(seg.atan, rot)) <= 0.0) &&
		(!veql(pts.a, seg.p1) || vdot(n, vrotate(seg.btan, rot)) <= 0.0))){
		contact_points(support_edge_segment(seg, n), support_edge_poly(poly, vneg(n)), pts, info);
	}
}

/* cpCollision.c:661-679 */
static __device__ void circle_poly(const ShapeView &circle, const ShapeView &poly, NInfo &info)
{
	CPts pts = gjk(circle, poly, info.id);
	if(pts.d <= circle.r + poly.r){
		V2 n = info.n = pts.n;
		push_contact(info, vadd(pts.a, vmul(n, circle.r)), vadd(pts.b, vmul(n, -poly.r)), 0ull);
	}
}

/* cpCollision.c:701-726.  Returns info for (a, b) after ordering by kind;
 * `flip` tells whether info.a is the second argument. */
static __device__ void collide(const ShapeView &a, const ShapeView &b, unsigned idIn, NInfo &info, int &flip)
{
	info.n = v2(0.0, 0.0);
	info.count = 0;
	info.id = idIn;
	flip = (a.kind > b.kind);
	const ShapeView &A = flip ? b : a;
	const ShapeView &B = flip ? a : b;
	switch(A.kind + B.kind*3){
		case 0: circle_circle(A, B, info); break;
		case 3: circle_segment(A, B, info); break;
		case 4: segment_segment(A, B, info); break;
		case 6: circle_poly(A, B, info); break;
		case 7: segment_poly(A, B, info); break;
		case 8: poly_poly(A, B, info); break;
		default: break;
	}
}
