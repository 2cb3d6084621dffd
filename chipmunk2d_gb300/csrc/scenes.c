/*
 * scenes.c -- seeded synthetic workloads, built only through the public
 * Chipmunk2D C API (cpSpaceNew, cpBodyNew, cpSpaceAddShape, ...).
 *
 * The same source is compiled into every library that implements the API
 * (the GPU drop-in, the CPU restatement used as the test oracle, and the
 * unmodified reference when it is available), so all of them receive
 * identical scenes.  Random numbers come from xoshiro256** seeded through
 * splitmix64; every derived quantity uses only +, -, *, / and sqrt, which
 * are correctly rounded under IEEE 754, so a scene is bit-identical on x86
 * and Arm hosts.  Normal variates use the Irwin-Hall sum of 12 uniforms
 * (mean 0, variance 1).
 *
 * Workloads (sizes scale with the `size` argument; defaults in brackets):
 *   1  pyramid: static ground segment (-600,-240)-(600,-240), r 0, u 1;
 *      `size` rows [14] of 30x30 boxes, row i has size-i boxes spaced 32
 *      apart centred on x=0 at y=-225+32i; mass 1, moment cpMomentForBox,
 *      u 0.6, e 0.
 *   2  circles: `size` [20000] circles r~U[0.5,2], mass pi r^2, u 0.7,
 *      e 0.1, uniform in a W x H box (1000x2000 at 20000, area scaled with
 *      the count) bounded by 4 static segments of radius 1; v~N(0,5)/axis.
 *   3  mixed: `size` [30000] dynamic bodies split evenly among circles
 *      r~U[0.5,3], convex polys (hull of 3..8 uniform points in a disk of
 *      radius U[1,4]) and segments (length U[2,8], radius 0.5); size/60
 *      chains [500] of 20 boxes 0.5x2 linked by pivot joints at shared
 *      endpoints, hung from static anchors along the top; square container
 *      (2000 at 30000) of 4 static segments r 1; u~U[0.3,1], e~U[0,0.3];
 *      v~N(0,5)/axis; density 1.
 *   4  tumble world: `size` bodies, 200x200 static box of 4 segments r 1,
 *      50/50 circles r~U[1,4] and 3-6-vertex hull polys of radius U[1,4],
 *      uniform positions, v~N(0,20)/axis, density 1, u 0.7, e 0.1.
 *   5  adjoint world: `size`/2 circles r~U[1,3] and `size`/2 boxes with
 *      sides U[2,6] at random orientations, dropped onto a static ground
 *      segment, density 1, u 0.7, e 0.1.
 *   6  joints and filters: pin-joint chains, slide-joint pairs and ropes,
 *      filtered free bodies (build_joints below).
 *   7  machines: motors, gears, ratchets, rotary springs and limits,
 *      grooves and damped springs (build_machines below).
 * Gravity is (0,-100); iterations are set per workload; the time step is
 * the caller's.
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "../../include/chipmunk_gb300.h"

typedef struct {
	uint64_t s[4];
} Rng;

static uint64_t splitmix64(uint64_t *x)
{
	uint64_t z = (*x += 0x9e3779b97f4a7c15ULL);
	z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
	z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
	return z ^ (z >> 31);
}

static void rng_seed(Rng *r, uint64_t seed)
{
	uint64_t x = seed;
	for(int i = 0; i < 4; i++) r->s[i] = splitmix64(&x);
}

static inline uint64_t rotl(const uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

static uint64_t rng_next(Rng *r)
{
	uint64_t *s = r->s;
	const uint64_t result = rotl(s[1] * 5, 7) * 9;
	const uint64_t t = s[1] << 17;
	s[2] ^= s[0];
	s[3] ^= s[1];
	s[1] ^= s[2];
	s[0] ^= s[3];
	s[2] ^= t;
	s[3] = rotl(s[3], 45);
	return result;
}

/* uniform in [0, 1) with 53 random bits */
static double rng_u01(Rng *r) { return (double)(rng_next(r) >> 11) * 0x1.0p-53; }
static double rng_uniform(Rng *r, double lo, double hi) { return lo + (hi - lo)*rng_u01(r); }
static int rng_int(Rng *r, int lo, int hi) { return lo + (int)(rng_next(r) % (uint64_t)(hi - lo + 1)); }

/* Irwin-Hall: sum of 12 U[0,1) minus 6 has mean 0 and variance 1. */
static double rng_normal(Rng *r)
{
	double s = 0.0;
	for(int i = 0; i < 12; i++) s += rng_u01(r);
	return s - 6.0;
}

/* A point uniform in [xlo,xhi) x [ylo,yhi), and a vector of normal
 * variates scaled by s.  The y coordinate is drawn first: C leaves the
 * order of two calls in one argument list unspecified (gcc evaluates them
 * right to left on x86-64 and left to right on AArch64), and the scenes
 * were first generated with y first, so every draw is sequenced here. */
static cpVect rng_point(Rng *r, double xlo, double xhi, double ylo, double yhi)
{
	double y = rng_uniform(r, ylo, yhi);
	double x = rng_uniform(r, xlo, xhi);
	return cpv(x, y);
}

static cpVect rng_normal2(Rng *r, double s)
{
	double y = s*rng_normal(r);
	double x = s*rng_normal(r);
	return cpv(x, y);
}

/* Point uniform in the disk of radius R by rejection from the square. */
static cpVect rng_in_disk(Rng *r, double R)
{
	for(;;){
		double x = rng_uniform(r, -1.0, 1.0), y = rng_uniform(r, -1.0, 1.0);
		if(x*x + y*y <= 1.0) return cpv(x*R, y*R);
	}
}

/* Random unit vector by rejection + normalisation (sqrt only). */
static cpVect rng_direction(Rng *r)
{
	for(;;){
		double x = rng_uniform(r, -1.0, 1.0), y = rng_uniform(r, -1.0, 1.0);
		double l2 = x*x + y*y;
		if(l2 > 1e-4 && l2 <= 1.0){ double l = sqrt(l2); return cpv(x/l, y/l); }
	}
}

/* 2^(6u) for u in [0,1) from repeated square roots of 2 (portable: only
 * sqrt and multiply), used for the log-uniform world sizes. */
static double pow64_frac(double u)
{
	double x = 6.0*u;
	double result = 1.0;
	int whole = (int)x;
	for(int i = 0; i < whole; i++) result *= 2.0;
	double frac = x - (double)whole;
	double root = 2.0;
	for(int k = 0; k < 40; k++){
		root = sqrt(root);
		frac *= 2.0;
		if(frac >= 1.0){ result *= root; frac -= 1.0; }
	}
	return result;
}

typedef struct cpxScene {
	cpSpace *space;
	int nbodies, cap_bodies;
	cpBody **bodies;          /* dynamic bodies in the order they were added */
	int nshapes, cap_shapes;
	cpShape **shapes;         /* every shape (static ones included), add order */
	int nconstraints, cap_constraints;
	cpConstraint **constraints;
	/* bodies whose type an edit round changed, with the mass and moment
	 * they get back when they turn dynamic again */
	cpBody *changed[4];
	double changedM[4], changedI[4];
	int nchanged;
} cpxScene;

static void push_ptr(void ***arr, int *n, int *cap, void *p)
{
	if(*n == *cap){
		*cap = (*cap ? 2*(*cap) : 64);
		*arr = (void **)realloc(*arr, sizeof(void *)*(size_t)(*cap));
	}
	(*arr)[(*n)++] = p;
}

static cpBody *add_body(cpxScene *sc, cpBody *body)
{
	cpSpaceAddBody(sc->space, body);
	push_ptr((void ***)&sc->bodies, &sc->nbodies, &sc->cap_bodies, body);
	return body;
}

static cpShape *add_shape(cpxScene *sc, cpShape *shape)
{
	cpSpaceAddShape(sc->space, shape);
	push_ptr((void ***)&sc->shapes, &sc->nshapes, &sc->cap_shapes, shape);
	return shape;
}

static cpConstraint *add_constraint(cpxScene *sc, cpConstraint *c)
{
	cpSpaceAddConstraint(sc->space, c);
	push_ptr((void ***)&sc->constraints, &sc->nconstraints, &sc->cap_constraints, c);
	return c;
}

static void add_wall(cpxScene *sc, cpVect a, cpVect b, double r, double u, double e)
{
	cpShape *s = cpSegmentShapeNew(cpSpaceGetStaticBody(sc->space), a, b, r);
	cpShapeSetFriction(s, u);
	cpShapeSetElasticity(s, e);
	add_shape(sc, s);
}

static void add_box_walls(cpxScene *sc, double hw, double hh, double r, double u, double e)
{
	add_wall(sc, cpv(-hw, -hh), cpv( hw, -hh), r, u, e);
	add_wall(sc, cpv( hw, -hh), cpv( hw,  hh), r, u, e);
	add_wall(sc, cpv( hw,  hh), cpv(-hw,  hh), r, u, e);
	add_wall(sc, cpv(-hw,  hh), cpv(-hw, -hh), r, u, e);
}

static void add_circle(cpxScene *sc, cpVect p, cpVect v, double r, double u, double e)
{
	double m = 3.14159265358979323846*r*r;
	cpBody *body = cpBodyNew(m, cpMomentForCircle(m, 0.0, r, cpvzero));
	cpBodySetPosition(body, p);
	cpBodySetVelocity(body, v);
	add_body(sc, body);
	cpShape *s = cpCircleShapeNew(body, r, cpvzero);
	cpShapeSetFriction(s, u);
	cpShapeSetElasticity(s, e);
	add_shape(sc, s);
}

/* Convex hull of k random points in a disk, recentred on its centroid. */
static void add_random_poly(cpxScene *sc, Rng *rng, cpVect p, cpVect v, int k, double R, double u, double e)
{
	cpVect pts[16], hull[16];
	for(int i = 0; i < k; i++) pts[i] = rng_in_disk(rng, R);
	int n = cpConvexHull(k, pts, hull, NULL, 0.0);
	if(n < 3){
		/* degenerate draw: fall back to a triangle of the disk radius */
		hull[0] = cpv(R, 0.0); hull[1] = cpv(-0.5*R, 0.8660254037844386*R); hull[2] = cpv(-0.5*R, -0.8660254037844386*R);
		n = 3;
	}
	cpVect c = cpCentroidForPoly(n, hull);
	for(int i = 0; i < n; i++) hull[i] = cpvsub(hull[i], c);
	double area = cpAreaForPoly(n, hull, 0.0);
	double m = area;
	cpBody *body = cpBodyNew(m, cpMomentForPoly(m, n, hull, cpvzero, 0.0));
	cpBodySetPosition(body, p);
	cpBodySetVelocity(body, v);
	add_body(sc, body);
	cpShape *s = cpPolyShapeNew(body, n, hull, cpTransformIdentity, 0.0);
	cpShapeSetFriction(s, u);
	cpShapeSetElasticity(s, e);
	add_shape(sc, s);
}

static void add_box(cpxScene *sc, cpVect p, cpVect v, double w, double h, double m, double u, double e)
{
	cpBody *body = cpBodyNew(m, cpMomentForBox(m, w, h));
	cpBodySetPosition(body, p);
	cpBodySetVelocity(body, v);
	add_body(sc, body);
	cpShape *s = cpBoxShapeNew(body, w, h, 0.0);
	cpShapeSetFriction(s, u);
	cpShapeSetElasticity(s, e);
	add_shape(sc, s);
}

static void build_pyramid(cpxScene *sc, int rows)
{
	add_wall(sc, cpv(-600.0, -240.0), cpv(600.0, -240.0), 0.0, 1.0, 0.0);
	for(int i = 0; i < rows; i++){
		for(int j = 0; j < rows - i; j++){
			double x = ((double)j - (double)(rows - 1 - i)*0.5)*32.0;
			double y = -225.0 + 32.0*(double)i;
			add_box(sc, cpv(x, y), cpvzero, 30.0, 30.0, 1.0, 0.6, 0.0);
		}
	}
}

static void build_circles(cpxScene *sc, int n, uint64_t seed)
{
	Rng rng; rng_seed(&rng, seed);
	double scale = sqrt((double)n/20000.0);
	double hw = 500.0*scale, hh = 1000.0*scale;
	add_box_walls(sc, hw, hh, 1.0, 0.7, 0.1);
	for(int i = 0; i < n; i++){
		double r = rng_uniform(&rng, 0.5, 2.0);
		cpVect p = rng_point(&rng, -hw + 3.0, hw - 3.0, -hh + 3.0, hh - 3.0);
		cpVect v = rng_normal2(&rng, 5.0);
		add_circle(sc, p, v, r, 0.7, 0.1);
	}
}

static void build_mixed(cpxScene *sc, int n, uint64_t seed)
{
	Rng rng; rng_seed(&rng, seed);
	double half = 1000.0*sqrt((double)n/30000.0);
	add_box_walls(sc, half, half, 1.0, 0.7, 0.1);

	/* chains: size/60 chains of 20 links 0.5 x 2, hung from the top */
	int chains = n/60;
	if(chains < 1) chains = 1;
	double top = half - 5.0;
	for(int c = 0; c < chains; c++){
		double x = -half + ((double)c + 0.5)*(2.0*half/(double)chains);
		cpBody *prev = cpSpaceGetStaticBody(sc->space);
		for(int l = 0; l < 20; l++){
			double m = 1.0;
			cpBody *link = cpBodyNew(m, cpMomentForBox(m, 0.5, 2.0));
			cpBodySetPosition(link, cpv(x, top - 2.0*(double)l - 1.0));
			add_body(sc, link);
			cpShape *s = cpBoxShapeNew(link, 0.5, 2.0, 0.0);
			cpShapeSetFriction(s, rng_uniform(&rng, 0.3, 1.0));
			cpShapeSetElasticity(s, rng_uniform(&rng, 0.0, 0.3));
			add_shape(sc, s);
			cpConstraint *j = cpPivotJointNew(prev, link, cpv(x, top - 2.0*(double)l));
			cpConstraintSetCollideBodies(j, cpFalse);
			add_constraint(sc, j);
			prev = link;
		}
	}

	double ylo = -half + 5.0, yhi = top - 45.0;
	for(int i = 0; i < n; i++){
		cpVect p = rng_point(&rng, -half + 5.0, half - 5.0, ylo, yhi);
		cpVect v = rng_normal2(&rng, 5.0);
		double u = rng_uniform(&rng, 0.3, 1.0);
		double e = rng_uniform(&rng, 0.0, 0.3);
		int kind = i % 3;
		if(kind == 0){
			add_circle(sc, p, v, rng_uniform(&rng, 0.5, 3.0), u, e);
		} else if(kind == 1){
			int k = rng_int(&rng, 3, 8);
			add_random_poly(sc, &rng, p, v, k, rng_uniform(&rng, 1.0, 4.0), u, e);
		} else {
			double len = rng_uniform(&rng, 2.0, 8.0);
			cpVect d = rng_direction(&rng);
			cpVect a = cpvmult(d, -0.5*len), b = cpvmult(d, 0.5*len);
			double m = cpAreaForSegment(a, b, 0.5);
			cpBody *body = cpBodyNew(m, cpMomentForSegment(m, a, b, 0.5));
			cpBodySetPosition(body, p);
			cpBodySetVelocity(body, v);
			add_body(sc, body);
			cpShape *s = cpSegmentShapeNew(body, a, b, 0.5);
			cpShapeSetFriction(s, u);
			cpShapeSetElasticity(s, e);
			add_shape(sc, s);
		}
	}
}

static void build_tumble(cpxScene *sc, int n, uint64_t seed)
{
	Rng rng; rng_seed(&rng, seed);
	add_box_walls(sc, 100.0, 100.0, 1.0, 0.7, 0.1);
	for(int i = 0; i < n; i++){
		cpVect p = rng_point(&rng, -94.0, 94.0, -94.0, 94.0);
		cpVect v = rng_normal2(&rng, 20.0);
		if(rng_u01(&rng) < 0.5){
			add_circle(sc, p, v, rng_uniform(&rng, 1.0, 4.0), 0.7, 0.1);
		} else {
			int k = rng_int(&rng, 3, 6);
			add_random_poly(sc, &rng, p, v, k, rng_uniform(&rng, 1.0, 4.0), 0.7, 0.1);
		}
	}
}

static void build_adjoint(cpxScene *sc, int n, uint64_t seed)
{
	Rng rng; rng_seed(&rng, seed);
	add_wall(sc, cpv(-120.0, 0.0), cpv(120.0, 0.0), 0.0, 0.7, 0.1);
	int half = n/2;
	for(int i = 0; i < n; i++){
		cpVect p = rng_point(&rng, -60.0, 60.0, 8.0, 120.0);
		cpVect v = rng_normal2(&rng, 1.0);
		if(i < half){
			add_circle(sc, p, v, rng_uniform(&rng, 1.0, 3.0), 0.7, 0.1);
		} else {
			double w = rng_uniform(&rng, 2.0, 6.0), h = rng_uniform(&rng, 2.0, 6.0);
			/* a random orientation: a box dropped flat lands on a kink of
			 * the contact geometry (tied support vertices) */
			double ang = rng_uniform(&rng, 0.0, 6.283185307179586);
			cpBody *body = cpBodyNew(w*h, cpMomentForBox(w*h, w, h));
			cpBodySetPosition(body, p);
			cpBodySetAngle(body, ang);
			cpBodySetVelocity(body, v);
			add_body(sc, body);
			cpShape *s = cpBoxShapeNew(body, w, h, 0.0);
			cpShapeSetFriction(s, 0.7);
			cpShapeSetElasticity(s, 0.1);
			add_shape(sc, s);
		}
	}
}

/* Workload 6, joints and filters: pin-joint chains, slide-joint pairs and
 * ropes, and free bodies sorted into collision categories.
 *   - size/40 chains [1] of 8 boxes 1 x 3 (mass 1) joined by pin joints
 *     between anchors 1.25 from their centres, 2.75 apart, so neighbouring
 *     links overlap by 0.25 and only their shared filter group keeps them
 *     from colliding; each chain hangs by a pin joint from a static anchor;
 *     every third chain's joints have a finite maxForce (the
 *     impulse clamp binds) and a finite maxBias; chains start swinging.
 *   - size/8 pairs of circles r~U[1,2] joined by a slide joint (min 3,
 *     max 6) at a separation U[1.5,8], so joints start below min, inside
 *     the band (n = 0) or beyond max, with v~N(0,15)/axis; every fourth has
 *     a finite maxForce; collideBodies off on every other pair.
 *   - size/8 circles hung from static anchors by slide joints (min 0,
 *     max U[4,12]), the anchors at the circles' start, so each rope is
 *     slack until the fall takes it past max.
 *   - `size` free bodies, circles r~U[1,3] and hull polys of radius U[1,3],
 *     category 1 << (i % 3); mask all categories, except every fifth body,
 *     which masks out the next category ((i + 1) % 3).
 * Container: square of half-size 60 sqrt(size/40) of 4 static segments r 1;
 * u~U[0.3,1], e~U[0,0.3], v~N(0,5)/axis unless stated; density 1. */
static void build_joints(cpxScene *sc, int n, uint64_t seed)
{
	Rng rng; rng_seed(&rng, seed);
	double half = 60.0*sqrt((double)n/40.0);
	if(half < 40.0) half = 40.0;
	add_box_walls(sc, half, half, 1.0, 0.7, 0.1);
	cpBody *ground = cpSpaceGetStaticBody(sc->space);
	double top = half - 4.0;

	int chains = n/40;
	if(chains < 1) chains = 1;
	for(int c = 0; c < chains; c++){
		double x = -half + ((double)c + 0.5)*(2.0*half/(double)chains);
		cpShapeFilter f = { (cpGroup)(uintptr_t)(c + 1), CP_ALL_CATEGORIES, CP_ALL_CATEGORIES };
		cpBody *prev = ground;
		cpVect prevAnchor = cpv(x, top);
		double vx0 = 10.0*rng_normal(&rng);
		for(int l = 0; l < 8; l++){
			double cy = top - 0.25 - 1.25 - 2.75*(double)l;
			cpBody *link = cpBodyNew(1.0, cpMomentForBox(1.0, 1.0, 3.0));
			cpBodySetPosition(link, cpv(x, cy));
			cpBodySetVelocity(link, cpv(vx0*(double)(l + 1)/8.0, 0.0));
			add_body(sc, link);
			cpShape *s = cpBoxShapeNew(link, 1.0, 3.0, 0.0);
			cpShapeSetFriction(s, rng_uniform(&rng, 0.3, 1.0));
			cpShapeSetElasticity(s, rng_uniform(&rng, 0.0, 0.3));
			cpShapeSetFilter(s, f);
			add_shape(sc, s);
			cpConstraint *j = cpPinJointNew(prev, link, prevAnchor, cpv(0.0, 1.25));
			if(c % 3 == 2){
				cpConstraintSetMaxForce(j, 3000.0);
				cpConstraintSetMaxBias(j, 40.0);
			}
			add_constraint(sc, j);
			prev = link;
			prevAnchor = cpv(0.0, -1.25);
		}
	}

	double lo = -half + 6.0, hi = half - 6.0;
	double ylo = -half + 6.0, yhi = top - 32.0;
	int pairs = n/8;
	for(int i = 0; i < pairs; i++){
		cpVect p = rng_point(&rng, lo, hi, ylo, yhi);
		cpVect d = rng_direction(&rng);
		double sep = rng_uniform(&rng, 1.5, 8.0);
		cpBody *bb[2];
		for(int k = 0; k < 2; k++){
			double r = rng_uniform(&rng, 1.0, 2.0), m = 3.14159265358979323846*r*r;
			cpBody *body = cpBodyNew(m, cpMomentForCircle(m, 0.0, r, cpvzero));
			cpBodySetPosition(body, cpvadd(p, cpvmult(d, k ? 0.5*sep : -0.5*sep)));
			cpBodySetVelocity(body, rng_normal2(&rng, 15.0));
			add_body(sc, body);
			cpShape *s = cpCircleShapeNew(body, r, cpvzero);
			cpShapeSetFriction(s, rng_uniform(&rng, 0.3, 1.0));
			cpShapeSetElasticity(s, rng_uniform(&rng, 0.0, 0.3));
			add_shape(sc, s);
			bb[k] = body;
		}
		cpConstraint *j = cpSlideJointNew(bb[0], bb[1], cpvzero, cpvzero, 3.0, 6.0);
		if(i % 4 == 3) cpConstraintSetMaxForce(j, 5000.0);
		if(i % 2 == 1) cpConstraintSetCollideBodies(j, cpFalse);
		add_constraint(sc, j);
	}

	int ropes = n/8;
	for(int i = 0; i < ropes; i++){
		cpVect p = rng_point(&rng, lo, hi, ylo, yhi);
		double r = rng_uniform(&rng, 1.0, 2.0), m = 3.14159265358979323846*r*r;
		cpBody *body = cpBodyNew(m, cpMomentForCircle(m, 0.0, r, cpvzero));
		cpBodySetPosition(body, p);
		cpBodySetVelocity(body, rng_normal2(&rng, 5.0));
		add_body(sc, body);
		cpShape *s = cpCircleShapeNew(body, r, cpvzero);
		cpShapeSetFriction(s, rng_uniform(&rng, 0.3, 1.0));
		cpShapeSetElasticity(s, rng_uniform(&rng, 0.0, 0.3));
		add_shape(sc, s);
		add_constraint(sc, cpSlideJointNew(ground, body, p, cpvzero, 0.0, rng_uniform(&rng, 4.0, 12.0)));
	}

	for(int i = 0; i < n; i++){
		cpVect p = rng_point(&rng, lo, hi, ylo, yhi);
		cpVect v = rng_normal2(&rng, 5.0);
		double u = rng_uniform(&rng, 0.3, 1.0), e = rng_uniform(&rng, 0.0, 0.3);
		if(i & 1){
			double R = rng_uniform(&rng, 1.0, 3.0);
			add_random_poly(sc, &rng, p, v, rng_int(&rng, 3, 6), R, u, e);
		}
		else add_circle(sc, p, v, rng_uniform(&rng, 1.0, 3.0), u, e);
		cpBitmask cat = (cpBitmask)1u << (i % 3);
		cpBitmask mask = (i % 5 == 0) ? (CP_ALL_CATEGORIES & ~((cpBitmask)1u << ((i + 1) % 3))) : CP_ALL_CATEGORIES;
		cpShapeFilter f = { CP_NO_GROUP, cat, mask };
		cpShapeSetFilter(sc->shapes[sc->nshapes - 1], f);
	}
}

/* ---- exported harness entry points (cpx_ prefix: workload plumbing, not
 * part of the Chipmunk2D API) ---- */

static void build_machines(cpxScene *sc, int n, uint64_t seed);

void *cpx_scene_build(int config, int size, unsigned long long seed)
{
	cpxScene *sc = (cpxScene *)calloc(1, sizeof(cpxScene));
	sc->space = cpSpaceNew();
	cpSpaceSetGravity(sc->space, cpv(0.0, -100.0));
	switch(config){
		case 1: build_pyramid(sc, size > 0 ? size : 14); cpSpaceSetIterations(sc->space, 10); break;
		case 2: build_circles(sc, size > 0 ? size : 20000, seed); cpSpaceSetIterations(sc->space, 10); break;
		case 3: build_mixed(sc, size > 0 ? size : 30000, seed); cpSpaceSetIterations(sc->space, 15); break;
		case 4: build_tumble(sc, size > 0 ? size : 121, seed); cpSpaceSetIterations(sc->space, 10); break;
		case 5: build_adjoint(sc, size > 0 ? size : 64, seed); cpSpaceSetIterations(sc->space, 10); break;
		case 6: build_joints(sc, size > 0 ? size : 400, seed); cpSpaceSetIterations(sc->space, 10); break;
		case 7: build_machines(sc, size > 0 ? size : 40, seed); cpSpaceSetIterations(sc->space, 10); break;
		default: cpSpaceFree(sc->space); free(sc); return NULL;
	}
	return sc;
}

/* Workload 7, machines: `size` [40] mechanisms on a grid, each built from
 * the remaining joints, with debris falling on them:
 *   - wheel W1 (circle r 2) on a pivot to the static body at its centre,
 *     driven by a simple motor (rate +-U[1,4]; maxForce 5e4 on odd
 *     mechanisms);
 *   - wheel W2 (circle r 1.5) on a pivot, geared to W1 (ratio U[0.5,2],
 *     phase 0) and held by a ratchet to the static body (ratchet 0.4);
 *   - bar B (8 x 1 box) on a pivot at one end, tied to W2 by a damped
 *     rotary spring (rest angle 0.3, stiffness 3000, damping 60) and to the
 *     static body by a rotary limit (-0.6, 0.9);
 *   - slider S (circle r 1) in a groove along B (x in [-3.5, 3.5] of B);
 *   - weight M (2 x 2 box) hanging from S by a damped spring (rest 5,
 *     stiffness 200, damping 8).
 * A mechanism's shapes share a filter group.  size/2 debris circles
 * r~U[0.5,1.5] fall from above with v~N(0,5)/axis; a ground segment and
 * side walls close the scene.  Friction 0.7, elasticity 0.1, density 1
 * except where masses are given. */
static void build_machines(cpxScene *sc, int n, uint64_t seed)
{
	Rng rng; rng_seed(&rng, seed);
	cpSpace *sp = sc->space;
	cpBody *ground = cpSpaceGetStaticBody(sp);
	int cols = (int)sqrt((double)n) + 1;
	double cell = 24.0;
	double half = 0.5*cell*(double)cols + 10.0;
	int rows = (n + cols - 1)/cols;
	double top = cell*(double)rows + 20.0;
	add_wall(sc, cpv(-half, 0.0), cpv(half, 0.0), 1.0, 0.7, 0.1);
	add_wall(sc, cpv(-half, 0.0), cpv(-half, top + 40.0), 1.0, 0.7, 0.1);
	add_wall(sc, cpv(half, 0.0), cpv(half, top + 40.0), 1.0, 0.7, 0.1);
	for(int i = 0; i < n; i++){
		double cx = -half + 10.0 + cell*((double)(i % cols) + 0.5);
		double cy = 12.0 + cell*(double)(i/cols);
		cpShapeFilter f = { (cpGroup)(uintptr_t)(1000 + i), CP_ALL_CATEGORIES, CP_ALL_CATEGORIES };
		cpShape *s;
		/* W1 */
		double m1 = 3.14159265358979323846*4.0;
		cpBody *w1 = add_body(sc, cpBodyNew(m1, cpMomentForCircle(m1, 0.0, 2.0, cpvzero)));
		cpBodySetPosition(w1, cpv(cx - 6.0, cy));
		s = add_shape(sc, cpCircleShapeNew(w1, 2.0, cpvzero)); cpShapeSetFriction(s, 0.7); cpShapeSetElasticity(s, 0.1); cpShapeSetFilter(s, f);
		add_constraint(sc, cpPivotJointNew(ground, w1, cpv(cx - 6.0, cy)));
		double rate = rng_uniform(&rng, 1.0, 4.0)*((i & 2) ? -1.0 : 1.0);
		cpConstraint *motor = add_constraint(sc, cpSimpleMotorNew(ground, w1, rate));
		if(i & 1) cpConstraintSetMaxForce(motor, 5e4);
		/* W2 */
		double m2 = 3.14159265358979323846*2.25;
		cpBody *w2 = add_body(sc, cpBodyNew(m2, cpMomentForCircle(m2, 0.0, 1.5, cpvzero)));
		cpBodySetPosition(w2, cpv(cx - 2.0, cy));
		s = add_shape(sc, cpCircleShapeNew(w2, 1.5, cpvzero)); cpShapeSetFriction(s, 0.7); cpShapeSetElasticity(s, 0.1); cpShapeSetFilter(s, f);
		add_constraint(sc, cpPivotJointNew(ground, w2, cpv(cx - 2.0, cy)));
		add_constraint(sc, cpGearJointNew(w1, w2, 0.0, rng_uniform(&rng, 0.5, 2.0)));
		add_constraint(sc, cpRatchetJointNew(ground, w2, 0.0, 0.4));
		/* B */
		cpBody *bar = add_body(sc, cpBodyNew(8.0, cpMomentForBox(8.0, 8.0, 1.0)));
		cpBodySetPosition(bar, cpv(cx + 4.0, cy + 2.0));
		s = add_shape(sc, cpBoxShapeNew(bar, 8.0, 1.0, 0.0)); cpShapeSetFriction(s, 0.7); cpShapeSetElasticity(s, 0.1); cpShapeSetFilter(s, f);
		add_constraint(sc, cpPivotJointNew(ground, bar, cpv(cx, cy + 2.0)));
		add_constraint(sc, cpDampedRotarySpringNew(w2, bar, 0.3, 3000.0, 60.0));
		add_constraint(sc, cpRotaryLimitJointNew(ground, bar, -0.6, 0.9));
		/* S */
		double ms = 3.14159265358979323846;
		cpBody *sl = add_body(sc, cpBodyNew(ms, cpMomentForCircle(ms, 0.0, 1.0, cpvzero)));
		cpBodySetPosition(sl, cpv(cx + 4.0 + rng_uniform(&rng, -3.0, 3.0), cy + 2.0));
		s = add_shape(sc, cpCircleShapeNew(sl, 1.0, cpvzero)); cpShapeSetFriction(s, 0.7); cpShapeSetElasticity(s, 0.1); cpShapeSetFilter(s, f);
		add_constraint(sc, cpGrooveJointNew(bar, sl, cpv(-3.5, 0.0), cpv(3.5, 0.0), cpvzero));
		/* M */
		cpBody *wt = add_body(sc, cpBodyNew(4.0, cpMomentForBox(4.0, 2.0, 2.0)));
		cpVect sp0 = cpBodyGetPosition(sl);
		cpBodySetPosition(wt, cpv(sp0.x, sp0.y - 5.0));
		s = add_shape(sc, cpBoxShapeNew(wt, 2.0, 2.0, 0.0)); cpShapeSetFriction(s, 0.7); cpShapeSetElasticity(s, 0.1); cpShapeSetFilter(s, f);
		add_constraint(sc, cpDampedSpringNew(sl, wt, cpvzero, cpvzero, 5.0, 200.0, 8.0));
	}
	for(int i = 0; i < n/2; i++){
		cpVect p = rng_point(&rng, -half + 3.0, half - 3.0, top, top + 30.0);
		cpVect v = rng_normal2(&rng, 5.0);
		add_circle(sc, p, v, rng_uniform(&rng, 0.5, 1.5), 0.7, 0.1);
	}
}

/* Whether one of b's shapes is within `margin` of a static shape's box.
 * A body that turns static while it touches a static body keeps that
 * arbiter forever (static pairs never age, cpSpaceStep.c:292-325); the
 * reference leaves its contacts in a contact buffer that is recycled after
 * the persistence window and, if the body turns dynamic again, warm-starts
 * from whatever that memory then holds.  The edit rounds keep clear of that
 * case. */
static int near_static(cpxScene *sc, cpBody *b, double margin)
{
	cpSpace *sp = sc->space;
	for(int k = 0; k < sc->nshapes; k++){
		cpShape *s = sc->shapes[k];
		if(cpShapeGetBody(s) != b || cpShapeGetSpace(s) != sp) continue;
		cpBB bb = cpShapeGetBB(s);
		bb.l -= margin; bb.b -= margin; bb.r += margin; bb.t += margin;
		for(int q = 0; q < sc->nshapes; q++){
			cpShape *o = sc->shapes[q];
			if(cpShapeGetSpace(o) != sp || cpBodyGetType(cpShapeGetBody(o)) != CP_BODY_TYPE_STATIC) continue;
			cpBB ob = cpShapeGetBB(o);
			if(bb.l <= ob.r && ob.l <= bb.r && bb.b <= ob.t && ob.b <= bb.t) return 1;
		}
	}
	return 0;
}

/* One round of edits between steps, the same calls in every
 * implementation (seeded by `seed` and `round`):
 *   - 1 in 16 single-shape dynamic bodies without constraints leave the
 *     space (shape first, then body);
 *   - as many new circles and polys (radius U[1,3]) enter near the top with
 *     v~N(0,10)/axis, plus one more;
 *   - one constraint (if any) leaves, and a pin joint joins a random
 *     dynamic body to its nearest dynamic neighbour (collideBodies off on
 *     odd rounds);
 *   - one dynamic body with shapes and no constraints, clear of static
 *     shapes (near_static), turns static and, on the next round, dynamic
 *     again with its mass and moment; one turns kinematic with a velocity,
 *     and dynamic on the next round.
 * Returns the number of edits. */
int cpx_scene_edit(void *h, int round, unsigned long long seed)
{
	cpxScene *sc = (cpxScene *)h;
	cpSpace *sp = sc->space;
	Rng rng; rng_seed(&rng, seed*1000003ull + (unsigned long long)round);
	int edits = 0;
	/* bodies that changed type last round go back to dynamic, with their
	 * mass and moment (cpBodySetType recomputes them from the shapes, and
	 * these shapes carry none) */
	for(int k = 0; k < sc->nchanged; k++){
		cpBody *b = sc->changed[k];
		if(cpBodyGetSpace(b) != sp) continue;
		cpBodySetType(b, CP_BODY_TYPE_DYNAMIC);
		cpBodySetMass(b, sc->changedM[k]);
		cpBodySetMoment(b, sc->changedI[k]);
		edits++;
	}
	sc->nchanged = 0;
	/* removals */
	int nb0 = sc->nbodies;
	for(int i = 0; i < nb0; i++){
		cpBody *b = sc->bodies[i];
		if(cpBodyGetSpace(b) != sp || rng_int(&rng, 0, 15) != 0) continue;
		cpShape *only = NULL; int nshape = 0, ncons = 0;
		for(int k = 0; k < sc->nshapes; k++) if(cpShapeGetBody(sc->shapes[k]) == b && cpShapeGetSpace(sc->shapes[k]) == sp){ only = sc->shapes[k]; nshape++; }
		for(int k = 0; k < sc->nconstraints; k++){
			cpConstraint *c = sc->constraints[k];
			if(cpConstraintGetSpace(c) == sp && (cpConstraintGetBodyA(c) == b || cpConstraintGetBodyB(c) == b)) ncons++;
		}
		if(nshape != 1 || ncons != 0) continue;
		cpSpaceRemoveShape(sp, only);
		cpSpaceRemoveBody(sp, b);
		edits += 2;
	}
	/* additions, dropped near the top of the scene's box of bodies */
	double lo = 1e30, hi = -1e30, top = -1e30;
	for(int i = 0; i < sc->nbodies; i++){
		cpBody *b = sc->bodies[i];
		if(cpBodyGetSpace(b) != sp) continue;
		cpVect p = cpBodyGetPosition(b);
		if(p.x < lo) lo = p.x;
		if(p.x > hi) hi = p.x;
		if(p.y > top) top = p.y;
	}
	if(lo > hi){ lo = -10.0; hi = 10.0; top = 0.0; }
	int adds = edits/2 + 1;
	for(int i = 0; i < adds; i++){
		cpVect p = rng_point(&rng, lo, hi, top + 4.0, top + 12.0);
		cpVect v = rng_normal2(&rng, 10.0);
		double u = rng_uniform(&rng, 0.3, 1.0), e = rng_uniform(&rng, 0.0, 0.3);
		if(i & 1){
			double R = rng_uniform(&rng, 1.0, 3.0);
			add_random_poly(sc, &rng, p, v, rng_int(&rng, 3, 6), R, u, e);
		} else {
			add_circle(sc, p, v, rng_uniform(&rng, 1.0, 3.0), u, e);
		}
		edits++;
	}
	/* constraints */
	int live = 0;
	for(int k = 0; k < sc->nconstraints; k++) live += (cpConstraintGetSpace(sc->constraints[k]) == sp);
	if(live > 0){
		int pick = rng_int(&rng, 0, live - 1);
		for(int k = 0; k < sc->nconstraints; k++){
			cpConstraint *c = sc->constraints[k];
			if(cpConstraintGetSpace(c) != sp) continue;
			if(pick-- == 0){ cpSpaceRemoveConstraint(sp, c); edits++; break; }
		}
	}
	/* the pin joint links a random dynamic body to its nearest dynamic
	 * neighbour, at their centres */
	cpBody *pa = NULL, *pb = NULL;
	for(int tries = 0; tries < 64 && !pa; tries++){
		cpBody *b = sc->bodies[rng_int(&rng, 0, sc->nbodies - 1)];
		if(cpBodyGetSpace(b) == sp && cpBodyGetType(b) == CP_BODY_TYPE_DYNAMIC) pa = b;
	}
	if(pa){
		cpVect q = cpBodyGetPosition(pa);
		double best = 1e300;
		for(int i = 0; i < sc->nbodies; i++){
			cpBody *b = sc->bodies[i];
			if(b == pa || cpBodyGetSpace(b) != sp || cpBodyGetType(b) != CP_BODY_TYPE_DYNAMIC) continue;
			double d = cpvdistsq(cpBodyGetPosition(b), q);
			if(d < best){ best = d; pb = b; }
		}
	}
	if(pa && pb){
		cpConstraint *j = cpPinJointNew(pa, pb, cpvzero, cpvzero);
		if(round & 1) cpConstraintSetCollideBodies(j, cpFalse);
		add_constraint(sc, j);
		edits++;
	}
	/* type changes: dynamic bodies in the space with shapes and without
	 * constraints (a joint between two bodies of infinite mass has no
	 * finite impulse) */
	for(int which = 0; which < 2; which++){
		for(int tries = 0; tries < 64; tries++){
			cpBody *b = sc->bodies[rng_int(&rng, 0, sc->nbodies - 1)];
			if(cpBodyGetSpace(b) != sp || cpBodyGetType(b) != CP_BODY_TYPE_DYNAMIC) continue;
			int has = 0, cons = 0;
			for(int k = 0; k < sc->nshapes && !has; k++) has = (cpShapeGetBody(sc->shapes[k]) == b && cpShapeGetSpace(sc->shapes[k]) == sp);
			for(int k = 0; k < sc->nconstraints; k++){
				cpConstraint *c = sc->constraints[k];
				cons += (cpConstraintGetSpace(c) == sp && (cpConstraintGetBodyA(c) == b || cpConstraintGetBodyB(c) == b));
			}
			if(!has || cons || (which == 0 && near_static(sc, b, 4.0))) continue;
			sc->changed[sc->nchanged] = b;
			sc->changedM[sc->nchanged] = cpBodyGetMass(b);
			sc->changedI[sc->nchanged] = cpBodyGetMoment(b);
			sc->nchanged++;
			if(which == 0){
				cpBodySetType(b, CP_BODY_TYPE_STATIC);
			} else {
				cpBodySetType(b, CP_BODY_TYPE_KINEMATIC);
				cpBodySetVelocity(b, rng_normal2(&rng, 3.0));
			}
			edits++;
			break;
		}
	}
	return edits;
}

cpSpace *cpx_scene_space(void *h) { return ((cpxScene *)h)->space; }
int cpx_scene_body_count(void *h) { return ((cpxScene *)h)->nbodies; }
int cpx_scene_shape_count(void *h) { return ((cpxScene *)h)->nshapes; }
int cpx_scene_constraint_count(void *h) { return ((cpxScene *)h)->nconstraints; }
cpBody *cpx_scene_body(void *h, int i) { return ((cpxScene *)h)->bodies[i]; }
cpShape *cpx_scene_shape(void *h, int i) { return ((cpxScene *)h)->shapes[i]; }
cpConstraint *cpx_scene_constraint(void *h, int i) { return ((cpxScene *)h)->constraints[i]; }

/* ---- spatial queries through the public API ----
 * nq seeded queries over the scene's extent, cycling through the kinds:
 * 0 cpSpacePointQuery, 1 cpSpacePointQueryNearest, 2 cpSpaceSegmentQuery,
 * 3 cpSpaceSegmentQueryFirst, 4 cpSpaceBBQuery, 5 cpShapePointQuery,
 * 6 cpShapeSegmentQuery, 7 cpSpaceShapeQuery.  Every callback and every
 * result is one record of 8 doubles: query, kind, shape (its index in the
 * scene, -1 none), point x, y, distance or alpha, gradient or normal x, y.
 * A shape query's callback gives [query, 7, shape, count, normal x, y, 0,
 * 0] and a record [query, 8, shape, pointA x, y, pointB x, y, distance]
 * per contact point; the query ends with [query, 9, its result, 0...].
 * Its probe is a scene shape or, every other time, a circle, box or
 * segment on a body of its own that is in no space.  Returns the record
 * count (records past cap are counted, not written). */
typedef struct QRec { double *out; int cap, n, qi, kind; } QRec;

static int shape_index_(const cpShape *s) { return s ? (int)(intptr_t)cpShapeGetUserData(s) - 1 : -1; }

static void q_put(QRec *r, int shape, cpVect p, double d, cpVect g)
{
	if(r->n < r->cap){
		double *o = r->out + 8*(size_t)r->n;
		o[0] = r->qi; o[1] = r->kind; o[2] = shape; o[3] = p.x; o[4] = p.y; o[5] = d; o[6] = g.x; o[7] = g.y;
	}
	r->n++;
}
static void q_point_cb(cpShape *s, cpVect p, cpFloat d, cpVect g, void *data) { q_put((QRec *)data, shape_index_(s), p, d, g); }
static void q_seg_cb(cpShape *s, cpVect p, cpVect n, cpFloat a, void *data) { q_put((QRec *)data, shape_index_(s), p, a, n); }
static void q_bb_cb(cpShape *s, void *data) { q_put((QRec *)data, shape_index_(s), cpvzero, 0.0, cpvzero); }
static void q_shape_cb(cpShape *s, cpContactPointSet *set, void *data)
{
	QRec *r = (QRec *)data;
	int idx = shape_index_(s);
	q_put(r, idx, cpv((double)set->count, set->normal.x), set->normal.y, cpvzero);
	int kind = r->kind;
	r->kind = 8;
	for(int i = 0; i < set->count; i++)
		q_put(r, idx, set->points[i].pointA, set->points[i].pointB.x, cpv(set->points[i].pointB.y, set->points[i].distance));
	r->kind = kind;
}

int cpx_scene_queries(void *h, int seed, int nq, double *out, int cap)
{
	cpxScene *sc = (cpxScene *)h;
	cpSpace *sp = sc->space;
	int *live = (int *)malloc(sizeof(int)*(size_t)(sc->nshapes > 0 ? sc->nshapes : 1));
	int nlive = 0;
	cpBB ext = cpBBNew(0.0, 0.0, 0.0, 0.0);
	for(int i = 0; i < sc->nshapes; i++){
		cpShape *s = sc->shapes[i];
		cpShapeSetUserData(s, (cpDataPointer)(intptr_t)(i + 1));
		if(cpShapeGetSpace(s) != sp) continue;
		cpBB bb = cpShapeGetBB(s);
		ext = nlive ? cpBBNew(bb.l < ext.l ? bb.l : ext.l, bb.b < ext.b ? bb.b : ext.b,
		                      bb.r > ext.r ? bb.r : ext.r, bb.t > ext.t ? bb.t : ext.t) : bb;
		live[nlive++] = i;
	}
	QRec rec = {out, cap, 0, 0, 0};
	Rng rng;
	rng_seed(&rng, (uint64_t)seed*0x9e3779b97f4a7c15ULL + 17u);
	double size = (ext.r - ext.l) > (ext.t - ext.b) ? (ext.r - ext.l) : (ext.t - ext.b);
	for(int qi = 0; qi < nq && nlive > 0; qi++){
		int kind = qi % 8;
		rec.qi = qi; rec.kind = kind;
		/* near a shape half of the time, anywhere in the extent otherwise */
		cpShape *target = sc->shapes[live[rng_int(&rng, 0, nlive - 1)]];
		cpBB tb = cpShapeGetBB(target);
		int nearShape = rng_int(&rng, 0, 1);
		double x0 = rng_uniform(&rng, ext.l, ext.r);
		double y0 = rng_uniform(&rng, ext.b, ext.t);
		cpVect p = nearShape ? cpv(0.5*(tb.l + tb.r) + rng_uniform(&rng, -2.0, 2.0), 0.5*(tb.b + tb.t) + rng_uniform(&rng, -2.0, 2.0)) : cpv(x0, y0);
		cpShapeFilter filter = CP_SHAPE_FILTER_ALL;
		if(rng_int(&rng, 0, 3) == 0){
			cpGroup grp = (cpGroup)rng_int(&rng, 0, 3);
			cpBitmask cat = (cpBitmask)1u << rng_int(&rng, 0, 3);
			cpBitmask mask = (cpBitmask)rng_int(&rng, 1, 15);
			filter = cpShapeFilterNew(grp, cat, mask);
		}
		double len = rng_uniform(&rng, 2.0, 0.25*size + 2.0);
		cpVect dir = rng_direction(&rng);
		cpVect q = cpvadd(p, cpvmult(dir, len));
		double r = rng_int(&rng, 0, 2) == 0 ? 0.0 : rng_uniform(&rng, 0.0, 1.5);
		switch(kind){
		case 0: {
			double md = rng_int(&rng, 0, 4) == 0 ? -0.25 : rng_uniform(&rng, 0.0, 4.0);
			cpSpacePointQuery(sp, p, md, filter, q_point_cb, &rec);
			break;
		}
		case 1: {
			cpPointQueryInfo info;
			double md = rng_uniform(&rng, 0.5, 20.0);
			cpShape *s = cpSpacePointQueryNearest(sp, p, md, filter, &info);
			q_put(&rec, s ? shape_index_(s) : -1, info.point, info.distance, info.gradient);
			break;
		}
		case 2:
			cpSpaceSegmentQuery(sp, p, q, r, filter, q_seg_cb, &rec);
			break;
		case 3: {
			cpSegmentQueryInfo info;
			cpShape *s = cpSpaceSegmentQueryFirst(sp, p, q, r, filter, &info);
			q_put(&rec, s ? shape_index_(s) : -1, info.point, info.alpha, info.normal);
			break;
		}
		case 4: {
			double hw = rng_uniform(&rng, 1.0, 30.0), hh = rng_uniform(&rng, 1.0, 30.0);
			cpSpaceBBQuery(sp, cpBBNew(p.x - hw, p.y - hh, p.x + hw, p.y + hh), filter, q_bb_cb, &rec);
			break;
		}
		case 5: {
			cpPointQueryInfo info;
			double d = cpShapePointQuery(target, p, &info);
			q_put(&rec, shape_index_(target), info.point, d, info.gradient);
			break;
		}
		case 6: {
			cpSegmentQueryInfo info;
			cpBool hit = cpShapeSegmentQuery(target, p, q, r, &info);
			q_put(&rec, hit ? shape_index_(target) : -1, info.point, info.alpha, info.normal);
			break;
		}
		default: {
			cpBool any;
			if((qi/8) % 2 == 0){
				/* a scene shape against the others */
				any = cpSpaceShapeQuery(sp, target, q_shape_cb, &rec);
			} else {
				cpBody *pb = cpBodyNew(1.0, 1.0);
				cpBodySetPosition(pb, p);
				cpBodySetAngle(pb, rng_uniform(&rng, 0.0, 6.0));
				cpShape *probe;
				int pk = (qi/16) % 3;
				if(pk == 0) probe = cpCircleShapeNew(pb, rng_uniform(&rng, 1.0, 6.0), cpvzero);
				else if(pk == 1) probe = cpBoxShapeNew(pb, rng_uniform(&rng, 2.0, 12.0), rng_uniform(&rng, 2.0, 12.0), rng_uniform(&rng, 0.0, 0.5));
				else probe = cpSegmentShapeNew(pb, cpv(-rng_uniform(&rng, 1.0, 8.0), 0.0), cpv(rng_uniform(&rng, 1.0, 8.0), 0.0), rng_uniform(&rng, 0.0, 1.0));
				cpShapeSetFilter(probe, filter);
				any = cpSpaceShapeQuery(sp, probe, q_shape_cb, &rec);
				cpShapeFree(probe);
				cpBodyFree(pb);
			}
			rec.kind = 9;
			q_put(&rec, (int)any, cpvzero, 0.0, cpvzero);
			break;
		}
		}
	}
	free(live);
	return rec.n;
}

/* Public-getter view of every dynamic body: position (transform origin),
 * velocity, angle, angular velocity, rotation -- 8 doubles per body. */
int cpx_scene_dump_public(void *h, double *out)
{
	cpxScene *sc = (cpxScene *)h;
	for(int i = 0; i < sc->nbodies; i++){
		cpBody *b = sc->bodies[i];
		cpVect p = cpBodyGetPosition(b), v = cpBodyGetVelocity(b), rot = cpBodyGetRotation(b);
		double *o = out + 8*i;
		o[0] = p.x; o[1] = p.y; o[2] = v.x; o[3] = v.y;
		o[4] = cpBodyGetAngle(b); o[5] = cpBodyGetAngularVelocity(b); o[6] = rot.x; o[7] = rot.y;
	}
	return sc->nbodies;
}

/* Sum over every body's arbiters of cpArbiterTotalImpulse, through the
 * public cpBodyEachArbiter iterator: 2 doubles per body. */
static void sum_impulse(cpBody *body, cpArbiter *arb, void *data)
{
	(void)body;
	cpVect j = cpArbiterTotalImpulse(arb);
	double *acc = (double *)data;
	acc[0] += j.x; acc[1] += j.y;
}

int cpx_scene_dump_impulses(void *h, double *out)
{
	cpxScene *sc = (cpxScene *)h;
	for(int i = 0; i < sc->nbodies; i++){
		out[2*i] = 0.0; out[2*i + 1] = 0.0;
		cpBodyEachArbiter(sc->bodies[i], sum_impulse, out + 2*i);
	}
	return sc->nbodies;
}

void cpx_scene_step(void *h, double dt, int steps)
{
	cpxScene *sc = (cpxScene *)h;
	for(int i = 0; i < steps; i++) cpSpaceStep(sc->space, dt);
}

void cpx_scene_free(void *h)
{
	cpxScene *sc = (cpxScene *)h;
	if(!sc) return;
	/* The space goes first: a space does not own its children, but freeing
	 * it may still read the bodies it holds. */
	cpSpaceFree(sc->space);
	for(int i = 0; i < sc->nconstraints; i++) cpConstraintFree(sc->constraints[i]);
	for(int i = 0; i < sc->nshapes; i++) cpShapeFree(sc->shapes[i]);
	for(int i = 0; i < sc->nbodies; i++) cpBodyFree(sc->bodies[i]);
	free(sc->bodies); free(sc->shapes); free(sc->constraints);
	free(sc);
}

/* Body counts of a batch of tumble worlds: round(8 * 64^u), u ~ U[0,1),
 * i.e. log-uniform in [8, 512]. */
void cpx_batch_sizes(int count, unsigned long long seed, int *out)
{
	Rng rng; rng_seed(&rng, seed);
	for(int i = 0; i < count; i++){
		double n = 8.0*pow64_frac(rng_u01(&rng));
		int k = (int)(n + 0.5);
		if(k < 8) k = 8;
		if(k > 512) k = 512;
		out[i] = k;
	}
}
