/*
 * cpg_query.cu -- spatial queries against a space on the device
 * (src/cpSpaceQuery.c:48-204).
 *
 * One thread answers one query.  In the exact-order mode it walks the
 * world's two AABB trees as the reference does: SubtreeQuery
 * (cpBBTree.c:355-365) for point and box queries, dynamic tree then
 * static tree; SubtreeSegmentQuery (cpBBTree.c:367-385) for segment
 * queries, static tree then dynamic tree, with the exit fraction t_exit
 * that the leaf callback returns (1 for the all-hits query, the running
 * best alpha for the first-hit query).  Recursion becomes an explicit
 * stack: a child pushed with the fraction its parent computed is entered
 * only if that fraction is still below t_exit when it is popped, which is
 * when the recursive version tests it.  Hits are written in visit order,
 * so the host calls the callbacks in the reference's order.
 *
 * In the coloured mode the dynamic tree is not re-indexed, so every
 * shape slot is tested, in slot order (removed slots have an empty
 * filter and are always rejected).  A shape is tested when its box meets
 * the query's box (point and box queries: the same shapes pass the final
 * test as through the tree's fattened boxes) or, for segment queries,
 * when the segment crosses its box grown by the query's radius: that
 * finds every shape the thick segment touches, where the tree walk, which
 * tests the boxes without the radius, can miss one that it grazes.
 *
 * Shape tests: cpShape.c:222-256 (point and segment query of a shape),
 * :298-318 (circle), :407-468 (segment), cpPolyShape.c:66-149 (polygon),
 * chipmunk_private.h:120-142 (CircleSegmentQuery), chipmunk.h:183-188
 * (closest point on a segment), cpBB.h:115-143 (box segment query).  They
 * read the world geometry the last step cached.
 */
#include <cuda_runtime.h>
#include "cpg_device.h"
#include "cpg_math.cuh"
#include "cpg_narrow.cuh"

#define CPG_QUERY_STACK 256
#define MAGIC_EPSILON 1e-5

__device__ __forceinline__ bool q_reject(const cpgSet &s, int g, const cpgQuery &q)
{
	unsigned long long grp = s.sgroup[g];
	return (grp != 0ull && grp == q.group) || (s.scat[g] & q.mask) == 0u || (q.cat & s.smask[g]) == 0u;
}

/* chipmunk.h:183-188 */
__device__ __forceinline__ V2 closest_on_segment(V2 p, V2 a, V2 b)
{
	V2 delta = vsub(a, b);
	double t = dclamp01(vdot(delta, vsub(p, b))/vlensq(delta));
	return vadd(b, vmul(delta, t));
}

/* chipmunk_private.h:120-142; hit: alpha < INFINITY */
__device__ void circle_segment_query(V2 center, double r1, V2 a, V2 b, double r2, cpgHit &h, int shape)
{
	V2 da = vsub(a, center);
	V2 db = vsub(b, center);
	double rsum = r1 + r2;
	double qa = vdot(da, da) - 2.0*vdot(da, db) + vdot(db, db);
	double qb = vdot(da, db) - vdot(da, da);
	double det = qb*qb - qa*(vdot(da, da) - rsum*rsum);
	if(det >= 0.0){
		double t = (-qb - sqrt(det))/(qa);
		if(0.0 <= t && t <= 1.0){
			V2 n = vnormalize(vlerp(da, db, t));
			V2 p = vsub(vlerp(a, b, t), vmul(n, r2));
			h.shape = shape; h.px = p.x; h.py = p.y; h.gx = n.x; h.gy = n.y; h.d = t;
		}
	}
}

/* The point query of shape g: distance, surface point and gradient. */
__device__ void shape_point_query(const cpgSet &s, int g, int vbase, V2 p, cpgHit &h, int shape)
{
	int kind = s.skind[g];
	double r = s.sr[g];
	V2 pt, grad;
	double dist;
	if(kind == CPG_CIRCLE){
		V2 tc = v2(s.w0x[g], s.w0y[g]);
		V2 delta = vsub(p, tc);
		double d = vlen(delta);
		double r_over_d = d > 0.0 ? r/d : r;
		pt = vadd(tc, vmul(delta, r_over_d));
		dist = d - r;
		grad = (d > MAGIC_EPSILON ? vmul(delta, 1.0/d) : v2(0.0, 1.0));
	} else if(kind == CPG_SEGMENT){
		V2 closest = closest_on_segment(p, v2(s.w0x[g], s.w0y[g]), v2(s.w1x[g], s.w1y[g]));
		V2 delta = vsub(p, closest);
		double d = vlen(delta);
		V2 gg = vmul(delta, 1.0/d);
		pt = (d != 0.0 ? vadd(closest, vmul(gg, r)) : closest);
		dist = d - r;
		/* the reference's small-distance gradient is the local normal */
		grad = (d > MAGIC_EPSILON ? gg : v2(s.snx[g], s.sny[g]));
	} else {
		int count = s.svcount[g], o = vbase + s.svoff[g];
		V2 v0 = v2(s.gvx[o + count - 1], s.gvy[o + count - 1]);
		double minDist = INFINITY;
		V2 closestPoint = v2(0.0, 0.0), closestNormal = v2(0.0, 0.0);
		bool outside = false;
		for(int i = 0; i < count; i++){
			V2 v1 = v2(s.gvx[o + i], s.gvy[o + i]);
			V2 n = v2(s.gnx[o + i], s.gny[o + i]);
			outside = outside || (vdot(n, vsub(p, v1)) > 0.0);
			V2 closest = closest_on_segment(p, v0, v1);
			double d = vlen(vsub(p, closest));
			if(d < minDist){
				minDist = d;
				closestPoint = closest;
				closestNormal = n;
			}
			v0 = v1;
		}
		double d = (outside ? minDist : -minDist);
		V2 gg = vmul(vsub(p, closestPoint), 1.0/d);
		pt = vadd(closestPoint, vmul(gg, r));
		dist = d - r;
		grad = (minDist > MAGIC_EPSILON ? gg : closestNormal);
	}
	h.shape = shape; h.px = pt.x; h.py = pt.y; h.d = dist; h.gx = grad.x; h.gy = grad.y;
}

/* The segment query of shape g (cpShape.c:238-256 with the kind's own
 * test); a hit sets h.shape.  h starts as the reference's blank info. */
__device__ void shape_segment_query(const cpgSet &s, int g, int vbase, V2 a, V2 b, double r2, cpgHit &h, int shape)
{
	h.shape = -1; h.px = b.x; h.py = b.y; h.gx = 0.0; h.gy = 0.0; h.d = 1.0;
	cpgHit nearest;
	shape_point_query(s, g, vbase, a, nearest, shape);
	if(nearest.d <= r2){
		V2 n = vnormalize(vsub(a, v2(nearest.px, nearest.py)));
		h.shape = shape; h.d = 0.0; h.gx = n.x; h.gy = n.y;
		return;
	}
	int kind = s.skind[g];
	if(kind == CPG_CIRCLE){
		circle_segment_query(v2(s.w0x[g], s.w0y[g]), s.sr[g], a, b, r2, h, shape);
	} else if(kind == CPG_SEGMENT){
		V2 ta = v2(s.w0x[g], s.w0y[g]), tb = v2(s.w1x[g], s.w1y[g]), n = v2(s.wnx[g], s.wny[g]);
		double d = vdot(vsub(ta, a), n);
		double r = s.sr[g] + r2;
		V2 flipped_n = (d > 0.0 ? vneg(n) : n);
		V2 seg_offset = vsub(vmul(flipped_n, r), a);
		V2 seg_a = vadd(ta, seg_offset);
		V2 seg_b = vadd(tb, seg_offset);
		V2 delta = vsub(b, a);
		if(vcross(delta, seg_a)*vcross(delta, seg_b) <= 0.0){
			double d_offset = d + (d > 0.0 ? -r : r);
			double ad = -d_offset;
			double bd = vdot(delta, n) - d_offset;
			if(ad*bd < 0.0){
				double t = ad/(ad - bd);
				V2 p = vsub(vlerp(a, b, t), vmul(flipped_n, r2));
				h.shape = shape; h.px = p.x; h.py = p.y; h.gx = flipped_n.x; h.gy = flipped_n.y; h.d = t;
			}
		} else if(r != 0.0){
			cpgHit h1, h2;
			h1.shape = -1; h1.px = b.x; h1.py = b.y; h1.gx = 0.0; h1.gy = 0.0; h1.d = 1.0;
			h2 = h1;
			circle_segment_query(ta, s.sr[g], a, b, r2, h1, shape);
			circle_segment_query(tb, s.sr[g], a, b, r2, h2, shape);
			h = (h1.d < h2.d) ? h1 : h2;
		}
	} else {
		int count = s.svcount[g], o = vbase + s.svoff[g];
		double r = s.sr[g];
		double rsum = r + r2;
		for(int i = 0; i < count; i++){
			V2 n = v2(s.gnx[o + i], s.gny[o + i]);
			double an = vdot(a, n);
			double d = an - vdot(v2(s.gvx[o + i], s.gvy[o + i]), n) - rsum;
			if(d < 0.0) continue;
			double bn = vdot(b, n);
			double t = d/dmax(an - bn, DBL_MIN);
			if(t < 0.0 || 1.0 < t) continue;
			V2 point = vlerp(a, b, t);
			double dt = vcross(n, point);
			int ip = o + (i - 1 + count)%count;
			double dtMin = vcross(n, v2(s.gvx[ip], s.gvy[ip]));
			double dtMax = vcross(n, v2(s.gvx[o + i], s.gvy[o + i]));
			if(dtMin <= dt && dt <= dtMax){
				V2 p = vsub(vlerp(a, b, t), vmul(n, r2));
				h.shape = shape; h.px = p.x; h.py = p.y; h.gx = n.x; h.gy = n.y; h.d = t;
			}
		}
		if(rsum > 0.0){
			for(int i = 0; i < count; i++){
				cpgHit c;
				c.shape = -1; c.px = b.x; c.py = b.y; c.gx = 0.0; c.gy = 0.0; c.d = 1.0;
				circle_segment_query(v2(s.gvx[o + i], s.gvy[o + i]), r, a, b, r2, c, shape);
				if(c.d < h.d) h = c;
			}
		}
	}
}

/* cpBB.h:115-143 */
__device__ double bb_segment_query(BB bb, V2 a, V2 b)
{
	V2 delta = vsub(b, a);
	double tmin = -INFINITY, tmax = INFINITY;
	if(delta.x == 0.0){
		if(a.x < bb.l || bb.r < a.x) return INFINITY;
	} else {
		double t1 = (bb.l - a.x)/delta.x;
		double t2 = (bb.r - a.x)/delta.x;
		tmin = dmax(tmin, dmin(t1, t2));
		tmax = dmin(tmax, dmax(t1, t2));
	}
	if(delta.y == 0.0){
		if(a.y < bb.b || bb.t < a.y) return INFINITY;
	} else {
		double t1 = (bb.b - a.y)/delta.y;
		double t2 = (bb.t - a.y)/delta.y;
		tmin = dmax(tmin, dmin(t1, t2));
		tmax = dmin(tmax, dmax(t1, t2));
	}
	if(tmin <= tmax && 0.0 <= tmax && tmin <= 1.0) return dmax(tmin, 0.0);
	return INFINITY;
}

/* Per-query output: all-hits queries append (up to cap, the count keeps
 * going so the host sees an overflow); nearest/first keep one record. */
struct QOut {
	cpgHit *hits;
	int cap;
	int n;
	cpgHit best;
};

__device__ __forceinline__ void q_emit(QOut &o, const cpgHit &h)
{
	if(o.n < o.cap) o.hits[o.n] = h;
	o.n++;
}

/* The leaf callbacks of cpSpaceQuery.c (NearestPointQuery :33-46,
 * NearestPointQueryNearest :61-74, SegmentQuery :105-121,
 * SegmentQueryFirst :138-152, BBQuery :183-193); returns the value the
 * reference's callback returns to the segment walk. */
__device__ double q_leaf(const cpgSet &s, const cpgWorld &W, const cpgQuery &q, int shape, QOut &o)
{
	int g = W.shapeOff + shape;
	if(q_reject(s, g, q)) return (q.kind == CPG_Q_SEGMENT_FIRST) ? o.best.d : 1.0;
	V2 a = v2(q.ax, q.ay), b = v2(q.bx, q.by);
	switch(q.kind){
	case CPG_Q_POINT: {
		cpgHit h;
		shape_point_query(s, g, W.vertOff, a, h, shape);
		if(h.d < q.r) q_emit(o, h);
		return 1.0;
	}
	case CPG_Q_POINT_NEAREST:
		if(!s.ssensor[g]){
			cpgHit h;
			shape_point_query(s, g, W.vertOff, a, h, shape);
			if(h.d < o.best.d) o.best = h;
		}
		return 1.0;
	case CPG_Q_SEGMENT: {
		cpgHit h;
		shape_segment_query(s, g, W.vertOff, a, b, q.r, h, shape);
		if(h.shape >= 0) q_emit(o, h);
		return 1.0;
	}
	case CPG_Q_SEGMENT_FIRST: {
		if(!s.ssensor[g]){
			cpgHit h;
			shape_segment_query(s, g, W.vertOff, a, b, q.r, h, shape);
			if(h.shape >= 0 && h.d < o.best.d) o.best = h;
		}
		return o.best.d;
	}
	default: {
		BB qb = bbnew(q.ax, q.ay, q.bx, q.by);
		if(bbintersects(qb, bbnew(s.bbl[g], s.bbb[g], s.bbr[g], s.bbt[g]))){
			cpgHit h;
			h.shape = shape; h.px = h.py = h.d = h.gx = h.gy = 0.0;
			q_emit(o, h);
		}
		return 1.0;
	}
	}
}

__device__ __forceinline__ BB q_node_bb(const cpgNode &n) { return bbnew(n.l, n.b, n.r, n.t); }

/* cpBBTree.c:355-365 as a walk with an explicit stack */
__device__ bool q_tree(const cpgSet &s, const cpgWorld &W, const cpgNode *nodes, int root, const cpgQuery &q, BB qb, QOut &o)
{
	if(root < 0) return true;
	int stack[CPG_QUERY_STACK];
	int sp = 0;
	stack[sp++] = root;
	for(int guard = 0; sp > 0; guard++){
		if(guard > 2*W.nodeCap + 2) return false;
		int n = stack[--sp];
		const cpgNode &nd = nodes[n];
		if(!bbintersects(q_node_bb(nd), qb)) continue;
		if(nd.obj >= 0){
			q_leaf(s, W, q, nd.obj, o);
		} else {
			if(sp + 2 > CPG_QUERY_STACK) return false;
			stack[sp++] = nd.B;
			stack[sp++] = nd.A;
		}
	}
	return true;
}

/* cpBBTree.c:367-385 as a walk with an explicit stack (the root is
 * entered without a box test, as the reference's entry does) */
__device__ bool q_tree_segment(const cpgSet &s, const cpgWorld &W, const cpgNode *nodes, int root, const cpgQuery &q,
                               double t_exit, QOut &o)
{
	if(root < 0) return true;
	int stack[CPG_QUERY_STACK];
	double tval[CPG_QUERY_STACK];
	int sp = 0;
	stack[sp] = root; tval[sp] = -INFINITY; sp++;
	V2 a = v2(q.ax, q.ay), b = v2(q.bx, q.by);
	for(int guard = 0; sp > 0; guard++){
		if(guard > 2*W.nodeCap + 2) return false;
		sp--;
		int n = stack[sp];
		if(!(tval[sp] < t_exit)) continue;
		const cpgNode &nd = nodes[n];
		if(nd.obj >= 0){
			t_exit = dmin(t_exit, q_leaf(s, W, q, nd.obj, o));
			continue;
		}
		int A = nd.A, B = nd.B;
		double t_a = bb_segment_query(q_node_bb(nodes[A]), a, b);
		double t_b = bb_segment_query(q_node_bb(nodes[B]), a, b);
		if(sp + 2 > CPG_QUERY_STACK) return false;
		/* the first child visited goes on top */
		if(t_a < t_b){
			stack[sp] = B; tval[sp] = t_b; sp++;
			stack[sp] = A; tval[sp] = t_a; sp++;
		} else {
			stack[sp] = A; tval[sp] = t_a; sp++;
			stack[sp] = B; tval[sp] = t_b; sp++;
		}
	}
	return true;
}

/* ---- the spatial hash's queries (cpSpaceHash.c:353-525), for a space on
 * cpSpaceUseSpatialHash: the cells of the box, each handle once by the
 * grid's stamp; the segment walks the cells it crosses in order ---- */
static __device__ __forceinline__ int qh_cell(int x, int y, int n)
{
	unsigned long long hx = (unsigned long long)(long long)x, hy = (unsigned long long)(long long)y;
	return (int)((hx*1640531513ull ^ hy*2654435789ull) % (unsigned long long)n);
}

static __device__ __forceinline__ int qh_floor(double f)
{
	int i = (int)f;
	return (f < 0.0 && f != (double)i) ? i - 1 : i;
}

/* which: 0 the dynamic grid, 1 the static one; skip: a shape passed over
 * without a stamp (the querying shape), -1 for none */
template <typename Leaf>
static __device__ void q_hash(const cpgSet &s, cpgNode *nodes, int which, BB qb, int skip, Leaf leaf)
{
	cpgTree &T = s.tree[0];
	const int *cells = s.gcells + (size_t)which*s.numcells;
	const int *bh = s.gbinHandle + (size_t)which*s.gbinCap, *bn = s.gbinNext + (size_t)which*s.gbinCap;
	unsigned stamp = T.gstamp[which];
	double dim = s.celldim;
	int l = qh_floor(qb.l/dim), r = qh_floor(qb.r/dim), b = qh_floor(qb.b/dim), t = qh_floor(qb.t/dim);
	for(int i = l; i <= r; i++){
		for(int j = b; j <= t; j++){
			int guard = 0;
			for(int k = cells[qh_cell(i, j, s.numcells)]; k >= 0 && guard <= s.gbinCap; k = bn[k], guard++){
				cpgNode &nd = nodes[bh[k]];
				if(nd.stamp == stamp || nd.obj == skip) continue;
				leaf(nd.obj);
				nd.stamp = stamp;
			}
		}
	}
	T.gstamp[which] = stamp + 1;
}

static __device__ double q_hash_segment(const cpgSet &s, const cpgWorld &W, cpgNode *nodes, int which, const cpgQuery &q,
                                        double t_exit, QOut &o)
{
	cpgTree &T = s.tree[0];
	const int *cells = s.gcells + (size_t)which*s.numcells;
	const int *bh = s.gbinHandle + (size_t)which*s.gbinCap, *bn = s.gbinNext + (size_t)which*s.gbinCap;
	unsigned stamp = T.gstamp[which];
	double inv = 1.0/s.celldim;
	V2 a = v2(q.ax*inv, q.ay*inv), b = v2(q.bx*inv, q.by*inv);
	int cell_x = qh_floor(a.x), cell_y = qh_floor(a.y);
	double t = 0.0;
	int x_inc, y_inc;
	double temp_v, temp_h;
	if(b.x > a.x){ x_inc = 1; temp_h = (floor(a.x + 1.0) - a.x); } else { x_inc = -1; temp_h = (a.x - floor(a.x)); }
	if(b.y > a.y){ y_inc = 1; temp_v = (floor(a.y + 1.0) - a.y); } else { y_inc = -1; temp_v = (a.y - floor(a.y)); }
	double dx = fabs(b.x - a.x), dy = fabs(b.y - a.y);
	double dt_dx = (dx != 0.0 ? 1.0/dx : CUDART_INF), dt_dy = (dy != 0.0 ? 1.0/dy : CUDART_INF);
	double next_h = (temp_h != 0.0 ? temp_h*dt_dx : dt_dx);
	double next_v = (temp_v != 0.0 ? temp_v*dt_dy : dt_dy);
	for(int guard = 0; t < t_exit; guard++){
		if(guard > (1 << 24)) break;
		double tc = 1.0;
		int bguard = 0;
		for(int k = cells[qh_cell(cell_x, cell_y, s.numcells)]; k >= 0 && bguard <= s.gbinCap; k = bn[k], bguard++){
			cpgNode &nd = nodes[bh[k]];
			if(nd.stamp == stamp) continue;
			tc = dmin(tc, q_leaf(s, W, q, nd.obj, o));
			nd.stamp = stamp;
		}
		t_exit = dmin(t_exit, tc);
		if(next_v < next_h){ cell_y += y_inc; t = next_v; next_v += dt_dy; }
		else { cell_x += x_inc; t = next_h; next_h += dt_dx; }
	}
	T.gstamp[which] = stamp + 1;
	return t_exit;
}

__device__ void query_one(const cpgSet &s, int w, const cpgQuery *queries, int i, cpgHit *hits, int cap,
                          int *counts, int brute, int *status);

__global__ void k_query(cpgSet s, int w, const cpgQuery *queries, int nq, cpgHit *hits, int cap,
                        int *counts, int brute, int *status)
{
	if(s.useHash){
		/* the grids' stamps order the queries: one thread, in call order */
		if(blockIdx.x != 0 || threadIdx.x != 0) return;
		for(int i = 0; i < nq; i++) query_one(s, w, queries, i, hits, cap, counts, brute, status);
		return;
	}
	int i = blockIdx.x*blockDim.x + threadIdx.x;
	if(i >= nq) return;
	query_one(s, w, queries, i, hits, cap, counts, brute, status);
}

__device__ void query_one(const cpgSet &s, int w, const cpgQuery *queries, int i, cpgHit *hits, int cap,
                          int *counts, int brute, int *status)
{
	const cpgWorld &W = s.world[w];
	const cpgTree &T = s.tree[w];
	const cpgNode *nodes = s.nodes + W.nodeOff;
	cpgQuery q = queries[i];
	QOut o;
	o.hits = hits + (size_t)i*cap;
	o.cap = cap;
	o.n = 0;
	/* the blank results of cpSpacePointQueryNearest / SegmentQueryFirst */
	o.best.shape = -1; o.best.pad = 0;
	o.best.px = 0.0; o.best.py = 0.0; o.best.gx = 0.0; o.best.gy = 0.0;
	o.best.d = q.r;
	if(q.kind == CPG_Q_SEGMENT_FIRST){ o.best.px = q.bx; o.best.py = q.by; o.best.d = 1.0; }
	bool ok = true;
	if(q.kind == CPG_Q_SHAPE_POINT || q.kind == CPG_Q_SHAPE_SEGMENT){
		/* one shape (cpShapePointQuery, cpShapeSegmentQuery) */
		int n = 0;
		if(q.pad >= 0 && q.pad < W.nshapes && cap > 0){
			int g = W.shapeOff + q.pad;
			cpgHit h;
			if(q.kind == CPG_Q_SHAPE_POINT) shape_point_query(s, g, W.vertOff, v2(q.ax, q.ay), h, q.pad);
			else shape_segment_query(s, g, W.vertOff, v2(q.ax, q.ay), v2(q.bx, q.by), q.r, h, q.pad);
			o.hits[0] = h;
			n = (h.shape >= 0) ? 1 : 0;
		}
		counts[i] = n;
		return;
	}
	if(brute){
		/* every slot, dynamic shapes' bodies first for point and box
		 * queries, static first for segment queries, as the trees are
		 * visited */
		bool segment = (q.kind == CPG_Q_SEGMENT || q.kind == CPG_Q_SEGMENT_FIRST);
		BB qb = (q.kind == CPG_Q_BB) ? bbnew(q.ax, q.ay, q.bx, q.by)
		        : bbnew(q.ax - dmax(q.r, 0.0), q.ay - dmax(q.r, 0.0), q.ax + dmax(q.r, 0.0), q.ay + dmax(q.r, 0.0));
		for(int pass = 0; pass < 2; pass++){
			bool wantStatic = segment ? (pass == 0) : (pass == 1);
			for(int k = 0; k < W.nshapes; k++){
				int g = W.shapeOff + k;
				bool isStatic = s.btype[W.bodyOff + s.sbody[g]] == CPG_STATIC;
				if(isStatic != wantStatic) continue;
				BB sb = bbnew(s.bbl[g], s.bbb[g], s.bbr[g], s.bbt[g]);
				if(segment){
					/* the box grown by the query's radius: every shape the
					 * thick segment touches is tested */
					double rr = dmax(q.r, 0.0);
					BB xb = bbnew(sb.l - rr, sb.b - rr, sb.r + rr, sb.t + rr);
					if(!(bb_segment_query(xb, v2(q.ax, q.ay), v2(q.bx, q.by)) < (q.kind == CPG_Q_SEGMENT_FIRST ? o.best.d : 1.0))) continue;
				} else if(!bbintersects(sb, qb)) continue;
				q_leaf(s, W, q, k, o);
			}
		}
	} else if(s.useHash){
		cpgNode *hn = s.nodes + W.nodeOff;
		if(q.kind == CPG_Q_SEGMENT || q.kind == CPG_Q_SEGMENT_FIRST){
			q_hash_segment(s, W, hn, 1, q, 1.0, o);
			q_hash_segment(s, W, hn, 0, q, q.kind == CPG_Q_SEGMENT_FIRST ? o.best.d : 1.0, o);
		} else {
			BB qb = (q.kind == CPG_Q_BB) ? bbnew(q.ax, q.ay, q.bx, q.by)
			        : bbnew(q.ax - dmax(q.r, 0.0), q.ay - dmax(q.r, 0.0), q.ax + dmax(q.r, 0.0), q.ay + dmax(q.r, 0.0));
			for(int which = 0; which < 2; which++)
				q_hash(s, hn, which, qb, -1, [&](int shape){ q_leaf(s, W, q, shape, o); });
		}
	} else if(q.kind == CPG_Q_SEGMENT || q.kind == CPG_Q_SEGMENT_FIRST){
		ok = q_tree_segment(s, W, nodes, T.statRoot, q, 1.0, o);
		if(ok) ok = q_tree_segment(s, W, nodes, T.dynRoot, q, q.kind == CPG_Q_SEGMENT_FIRST ? o.best.d : 1.0, o);
	} else {
		BB qb = (q.kind == CPG_Q_BB) ? bbnew(q.ax, q.ay, q.bx, q.by)
		        : bbnew(q.ax - dmax(q.r, 0.0), q.ay - dmax(q.r, 0.0), q.ax + dmax(q.r, 0.0), q.ay + dmax(q.r, 0.0));
		ok = q_tree(s, W, nodes, T.dynRoot, q, qb, o);
		if(ok) ok = q_tree(s, W, nodes, T.statRoot, q, qb, o);
	}
	if(!ok) atomicOr(status, 1);
	if(q.kind == CPG_Q_POINT_NEAREST || q.kind == CPG_Q_SEGMENT_FIRST){
		if(cap > 0) o.hits[0] = o.best;
		counts[i] = (o.best.shape >= 0) ? 1 : 0;
	} else {
		counts[i] = o.n;
	}
}

extern "C" int cpg_launch_query(const cpgSet *s, int world, const cpgQuery *queries, int nq, cpgHit *hits, int cap,
                                int *counts, int brute, int *status, void *stream)
{
	if(nq <= 0) return 0;
	k_query<<<(nq + 127)/128, 128, 0, (cudaStream_t)stream>>>(*s, world, queries, nq, hits, cap, counts, brute, status);
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

/* ---- shape queries (cpSpaceQuery.c:214-246) and cpShapesCollide ---- */

/* A probe's view for the narrow phase; planes holds its polygon planes as
 * four arrays of n (x, y of the points, then of the normals). */
__device__ ShapeView probe_view(const cpgProbe &p, const double *planes, int n)
{
	ShapeView v;
	v.kind = p.kind;
	v.r = p.r;
	v.p0 = v2(p.p0x, p.p0y); v.p1 = v2(p.p1x, p.p1y); v.n = v2(p.nx, p.ny);
	v.atan = v2(p.atx, p.aty); v.btan = v2(p.btx, p.bty);
	v.rot = v2(p.rotx, p.roty);
	v.bb = bbnew(p.bbl, p.bbb, p.bbr, p.bbt);
	v.hashid = p.hashid;
	v.count = p.count;
	v.vx = planes + p.voff; v.vy = planes + n + p.voff;
	v.nx = planes + 2*n + p.voff; v.ny = planes + 3*n + p.voff;
	return v;
}

/* cpShapesCollide(a, b): the contact set with a's side first */
__device__ void shapes_collide(const ShapeView &a, const ShapeView &b, cpgShapeHit &h)
{
	NInfo info;
	int flip;
	collide(a, b, 0u, info, flip);
	int count = info.count < 2 ? info.count : 2;
	h.count = count;
	V2 n = flip ? vneg(info.n) : info.n;
	h.nx = n.x; h.ny = n.y;
	for(int i = 0; i < 2; i++){
		h.ax[i] = h.ay[i] = h.bx[i] = h.by[i] = h.dist[i] = 0.0;
	}
	for(int i = 0; i < count; i++){
		V2 p1 = info.p1[i], p2 = info.p2[i];
		V2 pa = flip ? p2 : p1, pb = flip ? p1 : p2;
		h.ax[i] = pa.x; h.ay[i] = pa.y; h.bx[i] = pb.x; h.by[i] = pb.y;
		h.dist[i] = vdot(vsub(p2, p1), n);
	}
}

struct SQOut { cpgShapeHit *hits; int cap, n, any; };

/* ShapeQuery (cpSpaceQuery.c:214-228) on one leaf */
__device__ void shape_query_leaf(const cpgSet &s, const cpgWorld &W, const cpgProbe &p, const ShapeView &a, int shape, SQOut &o)
{
	int g = W.shapeOff + shape;
	unsigned long long grp = s.sgroup[g];
	bool reject = (p.group != 0ull && p.group == grp) || (p.cat & s.smask[g]) == 0u || (s.scat[g] & p.mask) == 0u;
	if(reject || shape == p.slot) return;
	NarrowCtx nc; nc.s = &s; nc.shapeBase = W.shapeOff; nc.bodyBase = W.bodyOff; nc.vertBase = W.vertOff;
	ShapeView b = load_shape(nc, shape);
	cpgShapeHit h;
	shapes_collide(a, b, h);
	if(h.count){
		h.shape = shape; h.sensor = s.ssensor[g]; h.pad = 0;
		if(o.n < o.cap) o.hits[o.n] = h;
		o.n++;
		o.any = !(p.sensor || s.ssensor[g]);
	}
}

__global__ void k_shape_query(cpgSet s, int w, cpgProbe p, const double *planes, int nplanes, int brute,
                              cpgShapeHit *hits, int cap, int *counts)
{
	if(blockIdx.x != 0 || threadIdx.x != 0) return;
	const cpgWorld &W = s.world[w];
	const cpgTree &T = s.tree[w];
	const cpgNode *nodes = s.nodes + W.nodeOff;
	ShapeView a = probe_view(p, planes, nplanes);
	BB qb = bbnew(p.bbl, p.bbb, p.bbr, p.bbt);
	SQOut o; o.hits = hits; o.cap = cap; o.n = 0; o.any = 0;
	bool ok = true;
	if(s.useHash){
		cpgNode *hn = s.nodes + W.nodeOff;
		for(int which = 0; which < 2; which++)
			q_hash(s, hn, which, qb, p.slot, [&](int shape){ shape_query_leaf(s, W, p, a, shape, o); });
	} else if(brute){
		for(int pass = 0; pass < 2; pass++){
			for(int k = 0; k < W.nshapes; k++){
				int g = W.shapeOff + k;
				bool isStatic = s.btype[W.bodyOff + s.sbody[g]] == CPG_STATIC;
				if(isStatic != (pass == 1)) continue;
				if(!bbintersects(bbnew(s.bbl[g], s.bbb[g], s.bbr[g], s.bbt[g]), qb)) continue;
				shape_query_leaf(s, W, p, a, k, o);
			}
		}
	} else {
		int roots[2] = { T.dynRoot, T.statRoot };
		for(int t = 0; t < 2 && ok; t++){
			if(roots[t] < 0) continue;
			int stack[CPG_QUERY_STACK];
			int sp = 0;
			stack[sp++] = roots[t];
			for(int guard = 0; sp > 0; guard++){
				if(guard > 2*W.nodeCap + 2){ ok = false; break; }
				int n = stack[--sp];
				const cpgNode &nd = nodes[n];
				if(!bbintersects(q_node_bb(nd), qb)) continue;
				if(nd.obj >= 0){
					shape_query_leaf(s, W, p, a, nd.obj, o);
				} else {
					if(sp + 2 > CPG_QUERY_STACK){ ok = false; break; }
					stack[sp++] = nd.B;
					stack[sp++] = nd.A;
				}
			}
		}
	}
	counts[0] = o.n;
	counts[1] = o.any;
	counts[2] = ok ? 0 : 1;
}

__global__ void k_shape_pair(const cpgProbe *probes, const double *planes, int nplanes, cpgShapeHit *hit, int *counts)
{
	if(blockIdx.x != 0 || threadIdx.x != 0) return;
	ShapeView a = probe_view(probes[0], planes, nplanes), b = probe_view(probes[1], planes, nplanes);
	cpgShapeHit h;
	shapes_collide(a, b, h);
	h.shape = -1; h.sensor = 0; h.pad = 0;
	*hit = h;
	counts[0] = h.count;
}

extern "C" int cpg_launch_shape_query(const cpgSet *s, int world, const cpgProbe *probe, const double *planes, int nplanes,
                                      int brute, cpgShapeHit *hits, int cap, int *counts, void *stream)
{
	k_shape_query<<<1, 32, 0, (cudaStream_t)stream>>>(*s, world, *probe, planes, nplanes, brute, hits, cap, counts);
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

extern "C" int cpg_launch_shape_pair(const cpgProbe *probes, const double *planes, int nplanes, cpgShapeHit *hit,
                                     int *counts, void *stream)
{
	k_shape_pair<<<1, 32, 0, (cudaStream_t)stream>>>(probes, planes, nplanes, hit, counts);
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
