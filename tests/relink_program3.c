/*
 * relink_program3.c -- an ordinary Chipmunk2D program (reference public API
 * only) that moves objects by hand between steps and re-indexes them: a
 * static platform body moved and turned (cpSpaceReindexStatic), a single
 * static shape's body moved (cpSpaceReindexShape), dynamic bodies
 * teleported (cpSpaceReindexShapesForBody, one of them with two shapes),
 * a shape given a large velocity before its re-index, a re-index of a
 * shape the space no longer holds, and shapes changed in place
 * (chipmunk_unsafe.h: radius, offset, endpoints, vertices).  Queries run
 * right after the re-indexes, before the next step, so they see the trees
 * as re-indexed.  It prints every body's state, the queries' results and
 * visit orders, and some shapes' boxes.  Built like relink_program.c.
 */
#include <stdio.h>
#include <stdlib.h>
#ifdef RELINK_REFERENCE_HEADERS
#include "chipmunk/chipmunk.h"
#include "chipmunk/chipmunk_unsafe.h"
#else
#include "chipmunk_gb300.h"
#endif

#define NB 20

static cpBody *bodies[NB + 1];
static cpShape *shapes[NB + 2];
static cpSpace *the_space;

/* a visit prints the shape and whether the space is locked (it is, in
 * queries and iterations: cpSpaceQuery.c:204, cpSpace.c:632) */
static void print_visit(cpShape *shape, void *data)
{
	(void)data;
	printf(" %d%s", (int)(size_t)cpShapeGetUserData(shape), cpSpaceIsLocked(the_space) ? "" : "u");
}

static void print_nearest(cpSpace *space, cpVect p)
{
	cpPointQueryInfo info;
	cpShape *s = cpSpacePointQueryNearest(space, p, 30.0, CP_SHAPE_FILTER_ALL, &info);
	printf("nearest %d %a %a %a %a %a\n", s ? (int)(size_t)cpShapeGetUserData(s) : -1,
	       info.point.x, info.point.y, info.distance, info.gradient.x, info.gradient.y);
}

static void print_ray(cpSpace *space, cpVect a, cpVect b)
{
	cpSegmentQueryInfo info;
	cpShape *s = cpSpaceSegmentQueryFirst(space, a, b, 0.5, CP_SHAPE_FILTER_ALL, &info);
	printf("ray %d %a %a %a %a %a\n", s ? (int)(size_t)cpShapeGetUserData(s) : -1,
	       info.point.x, info.point.y, info.normal.x, info.normal.y, info.alpha);
}

static void print_box(cpSpace *space, cpBB bb)
{
	printf("order box");
	cpSpaceBBQuery(space, bb, CP_SHAPE_FILTER_ALL, (cpSpaceBBQueryFunc)print_visit, NULL);
	printf("\n");
}

static void print_bb(const char *label, cpShape *s)
{
	cpBB bb = cpShapeGetBB(s);
	printf("%s %a %a %a %a\n", label, bb.l, bb.b, bb.r, bb.t);
}

int main(void)
{
	cpSpace *space = cpSpaceNew();
	the_space = space;
	cpSpaceSetIterations(space, 10);
	cpSpaceSetGravity(space, cpv(0.0, -100.0));

	cpShape *ground = cpSpaceAddShape(space, cpSegmentShapeNew(cpSpaceGetStaticBody(space), cpv(-300.0, 0.0), cpv(300.0, 0.0), 0.0));
	cpShapeSetFriction(ground, 1.0);
	cpShapeSetUserData(ground, (cpDataPointer)(size_t)100);

	/* a platform on a static body of its own, and a post on another */
	cpBody *plat = cpSpaceAddBody(space, cpBodyNewStatic());
	cpBodySetPosition(plat, cpv(-20.0, 60.0));
	cpShape *deck = cpSpaceAddShape(space, cpSegmentShapeNew(plat, cpv(-50.0, 0.0), cpv(50.0, 0.0), 2.0));
	cpShape *rail = cpSpaceAddShape(space, cpBoxShapeNew(plat, 8.0, 16.0, 0.0));
	cpShapeSetFriction(deck, 0.8); cpShapeSetFriction(rail, 0.8);
	cpShapeSetUserData(deck, (cpDataPointer)(size_t)101);
	cpShapeSetUserData(rail, (cpDataPointer)(size_t)102);
	cpBody *postBody = cpSpaceAddBody(space, cpBodyNewStatic());
	cpBodySetPosition(postBody, cpv(120.0, 10.0));
	cpShape *post = cpSpaceAddShape(space, cpCircleShapeNew(postBody, 8.0, cpvzero));
	cpShapeSetUserData(post, (cpDataPointer)(size_t)103);

	for(int i = 0; i < NB; i++){
		cpFloat m = 1.0 + 0.05*i;
		cpBody *b;
		cpShape *s;
		if(i % 2 == 0){
			b = cpBodyNew(m, cpMomentForCircle(m, 0.0, 4.0, cpvzero));
			s = cpCircleShapeNew(b, 4.0, cpvzero);
		} else {
			b = cpBodyNew(m, cpMomentForBox(m, 9.0, 7.0));
			s = cpBoxShapeNew(b, 9.0, 7.0, 0.0);
		}
		cpBodySetPosition(b, cpv(-70.0 + 11.0*(i % 10), 80.0 + 14.0*(i / 10)));
		cpSpaceAddBody(space, b);
		cpSpaceAddShape(space, s);
		cpShapeSetFriction(s, 0.6);
		cpShapeSetUserData(s, (cpDataPointer)(size_t)(i + 1));
		bodies[i] = b; shapes[i] = s;
	}
	/* a body with two shapes */
	cpBody *pair = cpSpaceAddBody(space, cpBodyNew(3.0, cpMomentForBox(3.0, 20.0, 6.0)));
	cpBodySetPosition(pair, cpv(60.0, 40.0));
	shapes[NB] = cpSpaceAddShape(space, cpBoxShapeNew(pair, 20.0, 6.0, 0.0));
	shapes[NB + 1] = cpSpaceAddShape(space, cpCircleShapeNew(pair, 5.0, cpv(10.0, 0.0)));
	cpShapeSetUserData(shapes[NB], (cpDataPointer)(size_t)50);
	cpShapeSetUserData(shapes[NB + 1], (cpDataPointer)(size_t)51);
	cpShapeSetFriction(shapes[NB], 0.7); cpShapeSetFriction(shapes[NB + 1], 0.7);
	bodies[NB] = pair;

	cpShape *gone = NULL;
	for(int step = 0; step < 200; step++){
		cpSpaceStep(space, 1.0/60.0);
		if(step == 49){
			/* the platform moves and turns under the bodies on it */
			cpBodySetPosition(plat, cpv(10.0, 45.0));
			cpBodySetAngle(plat, 0.15);
			cpSpaceReindexStatic(space);
			print_bb("bbdeck", deck);
			print_bb("bbrail", rail);
			print_nearest(space, cpv(10.0, 50.0));
			print_ray(space, cpv(-100.0, 44.0), cpv(100.0, 48.0));
			print_box(space, cpBBNew(-40.0, 30.0, 60.0, 70.0));
		}
		if(step == 79){
			/* teleports: a single body and the two-shape body */
			cpBodySetPosition(bodies[3], cpv(-150.0, 30.0));
			cpBodySetVelocity(bodies[3], cpv(0.0, 0.0));
			cpSpaceReindexShapesForBody(space, bodies[3]);
			cpBodySetPosition(pair, cpv(-100.0, 120.0));
			cpBodySetAngle(pair, 0.4);
			cpSpaceReindexShapesForBody(space, pair);
			print_nearest(space, cpv(-150.0, 31.0));
			print_box(space, cpBBNew(-160.0, 20.0, -80.0, 130.0));
			print_bb("bbpair0", shapes[NB]);
			print_bb("bbpair1", shapes[NB + 1]);
		}
		if(step == 99){
			/* one static shape moved on its own, a fast body re-indexed
			 * with its new velocity, and a no-op static re-index */
			cpBodySetPosition(postBody, cpv(-30.0, 8.0));
			cpSpaceReindexShape(space, post);
			cpBodySetVelocity(bodies[8], cpv(300.0, 120.0));
			cpSpaceReindexShape(space, shapes[8]);
			cpSpaceReindexStatic(space);
			print_ray(space, cpv(-60.0, 8.0), cpv(60.0, 8.0));
			print_box(space, cpBBNew(-50.0, 0.0, 0.0, 30.0));
		}
		if(step == 129){
			/* a shape leaves the space; its re-index only caches its box */
			gone = shapes[5];
			cpSpaceRemoveShape(space, gone);
			cpBodySetPosition(bodies[5], cpv(200.0, 200.0));
			cpSpaceReindexShape(space, gone);
			print_bb("bbgone", gone);
			cpSpaceReindexShapesForBody(space, bodies[6]);
		}
		if(step == 145){
			/* shapes changed in place, a static one re-indexed after */
			cpCircleShapeSetRadius(shapes[0], 6.0);
			cpCircleShapeSetOffset(shapes[2], cpv(1.0, 0.5));
			cpVect tri[4] = { cpv(-5.0, -4.0), cpv(6.0, -3.0), cpv(0.0, 5.0), cpv(-1.0, 0.0) };
			cpPolyShapeSetVerts(shapes[1], 4, tri, cpTransformIdentity);
			cpPolyShapeSetRadius(shapes[3], 0.5);
			cpSegmentShapeSetEndpoints(deck, cpv(-45.0, -1.0), cpv(48.0, 2.0));
			cpSegmentShapeSetRadius(deck, 2.5);
			cpSpaceReindexStatic(space);
			print_bb("bbdeck2", deck);
			print_box(space, cpBBNew(-60.0, 0.0, 60.0, 60.0));
		}
		if(step == 159){
			/* the platform back down, turned the other way */
			cpBodySetPosition(plat, cpv(-10.0, 20.0));
			cpBodySetAngle(plat, -0.1);
			cpSpaceReindexStatic(space);
			print_box(space, cpBBNew(-80.0, 0.0, 80.0, 60.0));
		}
	}
	printf("order each");
	cpSpaceEachShape(space, print_visit, NULL);
	printf("\n");
	printf("locked %d\n", (int)cpSpaceIsLocked(space));
	for(int i = 0; i <= NB; i++){
		cpVect p = cpBodyGetPosition(bodies[i]), v = cpBodyGetVelocity(bodies[i]);
		printf("%d %a %a %a %a %a %a\n", i, p.x, p.y, v.x, v.y, cpBodyGetAngle(bodies[i]), cpBodyGetAngularVelocity(bodies[i]));
	}
	print_nearest(space, cpv(0.0, 25.0));
	print_ray(space, cpv(-200.0, 5.0), cpv(200.0, 9.0));

	if(gone) cpShapeFree(gone);
	for(int i = 0; i < NB + 2; i++){
		if(shapes[i] == gone) continue;
		cpSpaceRemoveShape(space, shapes[i]);
		cpShapeFree(shapes[i]);
	}
	for(int i = 0; i <= NB; i++){ cpSpaceRemoveBody(space, bodies[i]); cpBodyFree(bodies[i]); }
	cpSpaceRemoveShape(space, deck); cpShapeFree(deck);
	cpSpaceRemoveShape(space, rail); cpShapeFree(rail);
	cpSpaceRemoveShape(space, post); cpShapeFree(post);
	cpSpaceRemoveShape(space, ground); cpShapeFree(ground);
	cpSpaceRemoveBody(space, plat); cpBodyFree(plat);
	cpSpaceRemoveBody(space, postBody); cpBodyFree(postBody);
	cpSpaceFree(space);
	return 0;
}
