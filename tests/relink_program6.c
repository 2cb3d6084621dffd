/*
 * relink_program6.c -- an ordinary Chipmunk2D program (reference public API
 * only) on the spatial hash (cpSpaceUseSpatialHash): the switch made after
 * the first shapes are in, a pile of boxes and balls, shapes removed and
 * added, a static body moved and re-indexed, a shape re-indexed by hand,
 * sleeping, and the queries (nearest, first hit, box, shape) with their
 * visit orders.  It prints the queries' results, the shape iteration order
 * and every body's state.  Built like relink_program.c.
 */
#include <stdio.h>
#include <stdlib.h>
#ifdef RELINK_REFERENCE_HEADERS
#include "chipmunk/chipmunk.h"
#else
#include "chipmunk_gb300.h"
#endif

#define MAXB 96

static cpBody *bodies[MAXB];
static cpShape *shapes[MAXB];
static int nbodies = 0;

static void print_visit(cpShape *shape, void *data)
{
	(void)data;
	printf(" %d", (int)(size_t)cpShapeGetUserData(shape));
}

static void print_shape_hit(cpShape *shape, cpContactPointSet *set, void *data)
{
	(void)data;
	printf(" %d:%d", (int)(size_t)cpShapeGetUserData(shape), set->count);
}

static cpFloat alphas[64];
static int nalphas;

static void print_segment_hit(cpShape *shape, cpVect point, cpVect normal, cpFloat alpha, void *data)
{
	(void)data; (void)point; (void)normal;
	printf(" %d", (int)(size_t)cpShapeGetUserData(shape));
	if(nalphas < 64) alphas[nalphas++] = alpha;
}

static void queries(cpSpace *space, int tag)
{
	cpPointQueryInfo pinfo;
	cpShape *s = cpSpacePointQueryNearest(space, cpv(-20.0 + tag, 30.0), 40.0, CP_SHAPE_FILTER_ALL, &pinfo);
	printf("nearest%d %d %a %a %a\n", tag, s ? (int)(size_t)cpShapeGetUserData(s) : -1, pinfo.point.x, pinfo.point.y, pinfo.distance);
	cpSegmentQueryInfo sinfo;
	s = cpSpaceSegmentQueryFirst(space, cpv(-150.0, 12.0), cpv(150.0, 30.0), 1.0, CP_SHAPE_FILTER_ALL, &sinfo);
	printf("ray%d %d %a %a %a\n", tag, s ? (int)(size_t)cpShapeGetUserData(s) : -1, sinfo.point.x, sinfo.point.y, sinfo.alpha);
	printf("order seg%d", tag);
	nalphas = 0;
	cpSpaceSegmentQuery(space, cpv(-120.0, 5.0), cpv(120.0, 45.0), 0.5, CP_SHAPE_FILTER_ALL, print_segment_hit, NULL);
	printf("\n");
	printf("alphas%d", tag);
	for(int i = 0; i < nalphas; i++) printf(" %a", alphas[i]);
	printf("\n");
	printf("order box%d", tag);
	cpSpaceBBQuery(space, cpBBNew(-60.0, 0.0, 40.0, 50.0), CP_SHAPE_FILTER_ALL, (cpSpaceBBQueryFunc)print_visit, NULL);
	printf("\n");
	printf("order shape%d", tag);
	cpSpaceShapeQuery(space, shapes[3], print_shape_hit, NULL);
	printf("\n");
}

static int add_box(cpSpace *space, cpVect p, cpFloat w, cpFloat h)
{
	cpBody *b = cpSpaceAddBody(space, cpBodyNew(1.0, cpMomentForBox(1.0, w, h)));
	cpBodySetPosition(b, p);
	cpShape *s = cpSpaceAddShape(space, cpBoxShapeNew(b, w, h, 0.0));
	cpShapeSetFriction(s, 0.7);
	cpShapeSetUserData(s, (cpDataPointer)(size_t)(nbodies + 1));
	bodies[nbodies] = b; shapes[nbodies] = s;
	return nbodies++;
}

static int add_ball(cpSpace *space, cpVect p, cpFloat r)
{
	cpBody *b = cpSpaceAddBody(space, cpBodyNew(1.0, cpMomentForCircle(1.0, 0.0, r, cpvzero)));
	cpBodySetPosition(b, p);
	cpShape *s = cpSpaceAddShape(space, cpCircleShapeNew(b, r, cpvzero));
	cpShapeSetFriction(s, 0.5);
	cpShapeSetElasticity(s, 0.2);
	cpShapeSetUserData(s, (cpDataPointer)(size_t)(nbodies + 1));
	bodies[nbodies] = b; shapes[nbodies] = s;
	return nbodies++;
}

int main(void)
{
	cpSpace *space = cpSpaceNew();
	cpSpaceSetIterations(space, 10);
	cpSpaceSetGravity(space, cpv(0.0, -100.0));
	cpShape *ground = cpSpaceAddShape(space, cpSegmentShapeNew(cpSpaceGetStaticBody(space), cpv(-200.0, 0.0), cpv(200.0, 0.0), 1.0));
	cpShapeSetFriction(ground, 1.0);
	cpShapeSetUserData(ground, (cpDataPointer)(size_t)100);
	cpBody *wallBody = cpSpaceAddBody(space, cpBodyNewStatic());
	cpBodySetPosition(wallBody, cpv(90.0, 20.0));
	cpShape *wall = cpSpaceAddShape(space, cpBoxShapeNew(wallBody, 6.0, 40.0, 0.0));
	cpShapeSetUserData(wall, (cpDataPointer)(size_t)101);
	for(int k = 0; k < 4; k++) add_box(space, cpv(-60.0 + 11.0*k, 6.0), 10.0, 10.0);

	/* the switch, with shapes already in both indices */
	cpSpaceUseSpatialHash(space, 12.0, 1000);

	for(int i = 0; i < 5; i++)
		for(int j = 0; j < 5 - i; j++) add_box(space, cpv(-20.0 + 10.5*j + 5.0*i, 6.0 + 10.2*(i + 1)), 10.0, 10.0);
	for(int k = 0; k < 12; k++) add_ball(space, cpv(-100.0 + 17.0*k, 70.0 + 6.0*(k % 4)), 2.0 + 0.5*(k % 5));
	cpSpaceSetSleepTimeThreshold(space, 0.4);

	for(int step = 0; step < 360; step++){
		cpSpaceStep(space, 1.0/60.0);
		if(step == 60) queries(space, 1);
		if(step == 90){
			/* a ball and a box leave; two balls come */
			cpSpaceRemoveShape(space, shapes[25]); cpSpaceRemoveBody(space, bodies[25]);
			cpShapeFree(shapes[25]); cpBodyFree(bodies[25]); shapes[25] = NULL; bodies[25] = NULL;
			cpSpaceRemoveShape(space, shapes[6]); cpSpaceRemoveBody(space, bodies[6]);
			cpShapeFree(shapes[6]); cpBodyFree(bodies[6]); shapes[6] = NULL; bodies[6] = NULL;
			add_ball(space, cpv(10.0, 90.0), 3.0);
			add_ball(space, cpv(60.0, 95.0), 4.0);
		}
		if(step == 150){
			/* the wall moves and the static index is hashed again */
			cpBodySetPosition(wallBody, cpv(70.0, 22.0));
			cpSpaceReindexStatic(space);
			cpBodySetPosition(bodies[30], cpv(-130.0, 40.0));
			cpSpaceReindexShape(space, shapes[30]);
			queries(space, 2);
		}
		if(step == 300) queries(space, 3);
	}
	printf("order each");
	cpSpaceEachShape(space, print_visit, NULL);
	printf("\n");
	printf("order sleep");
	for(int i = 0; i < nbodies; i++) printf(" %d", bodies[i] ? (int)cpBodyIsSleeping(bodies[i]) : -1);
	printf("\n");
	for(int i = 0; i < nbodies; i++){
		if(!bodies[i]) continue;
		cpVect p = cpBodyGetPosition(bodies[i]), v = cpBodyGetVelocity(bodies[i]);
		printf("%d %a %a %a %a %a %a\n", i, p.x, p.y, v.x, v.y, cpBodyGetAngle(bodies[i]), cpBodyGetAngularVelocity(bodies[i]));
	}
	for(int i = 0; i < nbodies; i++){
		if(!bodies[i]) continue;
		cpSpaceRemoveShape(space, shapes[i]); cpShapeFree(shapes[i]);
		cpSpaceRemoveBody(space, bodies[i]); cpBodyFree(bodies[i]);
	}
	cpSpaceRemoveShape(space, wall); cpShapeFree(wall);
	cpSpaceRemoveBody(space, wallBody); cpBodyFree(wallBody);
	cpSpaceRemoveShape(space, ground); cpShapeFree(ground);
	cpSpaceFree(space);
	return 0;
}
