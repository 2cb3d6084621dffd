/*
 * relink_program4.c -- an ordinary Chipmunk2D program (reference public API
 * only) with sleeping turned on.  A pyramid, a chain of boxes joined by
 * pivots lying on the ground and a few loose bodies come to rest and fall
 * asleep; a body on a moving kinematic platform stays awake.  Then the
 * program wakes them in every way the API offers: a new body dropped on
 * the sleeping pyramid, an impulse, a joint setter, a shape setter,
 * cpBodyActivateStatic on the ground, cpSpaceSetGravity, removing a
 * sleeping body's shape and body, and it puts bodies to sleep by hand
 * (cpBodySleep, cpBodySleepWithGroup).  It prints which bodies sleep, the
 * body iteration order (sleeping components last), a sleeping body's
 * arbiters, queries, and every body's final state.  Built like
 * relink_program.c.
 */
#include <stdio.h>
#include <stdlib.h>
#ifdef RELINK_REFERENCE_HEADERS
#include "chipmunk/chipmunk.h"
#else
#include "chipmunk_gb300.h"
#endif

#define MAXB 64

static cpBody *bodies[MAXB];
static cpShape *shapes[MAXB];
static int nbodies = 0;

static int add_box(cpSpace *space, cpVect p, cpFloat w, cpFloat h, cpFloat m)
{
	cpBody *b = cpSpaceAddBody(space, cpBodyNew(m, cpMomentForBox(m, w, h)));
	cpBodySetPosition(b, p);
	cpShape *s = cpSpaceAddShape(space, cpBoxShapeNew(b, w, h, 0.0));
	cpShapeSetFriction(s, 0.8);
	cpBodySetUserData(b, (cpDataPointer)(size_t)(nbodies + 1));
	cpShapeSetUserData(s, (cpDataPointer)(size_t)(nbodies + 1));
	bodies[nbodies] = b; shapes[nbodies] = s;
	return nbodies++;
}

static int add_ball(cpSpace *space, cpVect p, cpFloat r)
{
	cpBody *b = cpSpaceAddBody(space, cpBodyNew(1.5, cpMomentForCircle(1.5, 0.0, r, cpvzero)));
	cpBodySetPosition(b, p);
	cpShape *s = cpSpaceAddShape(space, cpCircleShapeNew(b, r, cpvzero));
	cpShapeSetFriction(s, 0.7);
	cpShapeSetElasticity(s, 0.1);
	cpBodySetUserData(b, (cpDataPointer)(size_t)(nbodies + 1));
	cpShapeSetUserData(s, (cpDataPointer)(size_t)(nbodies + 1));
	bodies[nbodies] = b; shapes[nbodies] = s;
	return nbodies++;
}

static void print_body_id(cpBody *body, void *data)
{
	(void)data;
	printf(" %d", (int)(size_t)cpBodyGetUserData(body));
}

static void print_arb(cpBody *body, cpArbiter *arb, void *data)
{
	(void)data;
	cpBody *a, *b;
	cpArbiterGetBodies(arb, &a, &b);
	(void)body;
	printf(" %d:%d:%d", (int)(size_t)cpBodyGetUserData(a), (int)(size_t)cpBodyGetUserData(b), cpArbiterGetCount(arb));
}

static void print_sleep(int step)
{
	printf("order sleep%d", step);
	for(int i = 0; i < nbodies; i++) printf(" %d", bodies[i] ? (int)cpBodyIsSleeping(bodies[i]) : -1);
	printf("\n");
}

static void print_order(cpSpace *space, int step)
{
	printf("order bodies%d", step);
	cpSpaceEachBody(space, print_body_id, NULL);
	printf("\n");
}

int main(void)
{
	cpSpace *space = cpSpaceNew();
	cpSpaceSetIterations(space, 10);
	cpSpaceSetGravity(space, cpv(0.0, -100.0));
	cpSpaceSetSleepTimeThreshold(space, 0.5);

	cpBody *staticBody = cpSpaceGetStaticBody(space);
	cpBodySetUserData(staticBody, (cpDataPointer)(size_t)0);
	cpShape *ground = cpSpaceAddShape(space, cpSegmentShapeNew(staticBody, cpv(-400.0, 0.0), cpv(400.0, 0.0), 0.0));
	cpShapeSetFriction(ground, 1.0);

	/* a pyramid of 5 rows */
	for(int i = 0; i < 5; i++)
		for(int j = 0; j < 5 - i; j++) add_box(space, cpv(-150.0 + (j - (4 - i)/2.0)*21.0, 10.0 + 20.5*i), 20.0, 20.0, 1.0);
	/* a chain of 6 boxes on the ground, joined at their ends */
	int chain0 = nbodies;
	for(int k = 0; k < 6; k++) add_box(space, cpv(20.0 + 16.0*k, 2.5), 15.0, 5.0, 0.5);
	cpConstraint *links[5];
	for(int k = 0; k < 5; k++){
		links[k] = cpSpaceAddConstraint(space, cpPivotJointNew(bodies[chain0 + k], bodies[chain0 + k + 1], cpv(28.0 + 16.0*k, 2.5)));
	}
	/* loose balls */
	int ball0 = nbodies;
	for(int k = 0; k < 4; k++) add_ball(space, cpv(180.0 + 30.0*k, 20.0 + 10.0*k), 5.0 + k);
	/* a box riding a kinematic platform: never sleeps */
	cpBody *plat = cpSpaceAddBody(space, cpBodyNewKinematic());
	cpBodySetUserData(plat, (cpDataPointer)(size_t)99);
	cpBodySetPosition(plat, cpv(-300.0, 40.0));
	cpBodySetVelocity(plat, cpv(2.0, 0.0));
	cpShape *platShape = cpSpaceAddShape(space, cpBoxShapeNew(plat, 60.0, 6.0, 0.0));
	cpShapeSetFriction(platShape, 1.0);
	int rider = add_box(space, cpv(-300.0, 53.0), 10.0, 10.0, 1.0);

	cpBody *dropped = NULL;
	for(int step = 0; step < 600; step++){
		cpSpaceStep(space, 1.0/60.0);
		if(step == 150){
			print_sleep(step);
			print_order(space, step);
			printf("order arbs");
			cpBodyEachArbiter(bodies[2], print_arb, NULL);
			printf("\n");
			cpPointQueryInfo info;
			cpShape *s = cpSpacePointQueryNearest(space, cpv(-150.0, 5.0), 30.0, CP_SHAPE_FILTER_ALL, &info);
			printf("nearest %d %a %a %a\n", s ? (int)(size_t)cpShapeGetUserData(s) : -1, info.point.x, info.point.y, info.distance);
		}
		if(step == 160){
			/* a ball dropped on the sleeping pyramid wakes it on contact */
			dropped = bodies[add_ball(space, cpv(-150.0, 160.0), 6.0)];
		}
		if(step == 200) print_sleep(step);
		if(step == 260){
			print_sleep(step);
			/* an impulse wakes the chain; a joint setter wakes what it joins */
			cpBodyApplyImpulseAtWorldPoint(bodies[chain0 + 2], cpv(0.0, 40.0), cpBodyGetPosition(bodies[chain0 + 2]));
			cpPivotJointSetAnchorB(links[4], cpPivotJointGetAnchorB(links[4]));
			cpShapeSetFriction(shapes[ball0], 0.7);
		}
		if(step == 330){
			print_sleep(step);
			print_order(space, step);
			/* the ground wakes whatever sleeps on it */
			cpBodyActivateStatic(staticBody, NULL);
			print_sleep(331);
		}
		if(step == 400){
			print_sleep(step);
			/* put a ball to sleep in the air, and another into its group */
			cpBodySetPosition(bodies[ball0 + 1], cpv(230.0, 120.0));
			cpBodySetVelocity(bodies[ball0 + 1], cpvzero);
			cpBodySleep(bodies[ball0 + 1]);
			cpBodySetPosition(bodies[ball0 + 2], cpv(260.0, 120.0));
			cpBodySleepWithGroup(bodies[ball0 + 2], bodies[ball0 + 1]);
			print_sleep(401);
			print_order(space, 401);
		}
		if(step == 460){
			print_sleep(step);
			/* new gravity wakes sleeping components */
			cpSpaceSetGravity(space, cpv(0.0, -120.0));
			print_sleep(461);
		}
		if(step == 540){
			print_sleep(step);
			/* a sleeping box leaves the space */
			int victim = 1;
			cpSpaceRemoveShape(space, shapes[victim]);
			cpSpaceRemoveBody(space, bodies[victim]);
			cpShapeFree(shapes[victim]);
			cpBodyFree(bodies[victim]);
			bodies[victim] = NULL; shapes[victim] = NULL;
			print_sleep(541);
		}
	}
	print_sleep(600);
	print_order(space, 600);
	for(int i = 0; i < nbodies; i++){
		if(!bodies[i]) continue;
		cpVect p = cpBodyGetPosition(bodies[i]), v = cpBodyGetVelocity(bodies[i]);
		printf("%d %a %a %a %a %a %a\n", i, p.x, p.y, v.x, v.y, cpBodyGetAngle(bodies[i]), cpBodyGetAngularVelocity(bodies[i]));
	}
	(void)dropped; (void)rider;

	for(int k = 0; k < 5; k++){ cpSpaceRemoveConstraint(space, links[k]); cpConstraintFree(links[k]); }
	for(int i = 0; i < nbodies; i++){
		if(!bodies[i]) continue;
		cpSpaceRemoveShape(space, shapes[i]); cpShapeFree(shapes[i]);
		cpSpaceRemoveBody(space, bodies[i]); cpBodyFree(bodies[i]);
	}
	cpSpaceRemoveShape(space, platShape); cpShapeFree(platShape);
	cpSpaceRemoveBody(space, plat); cpBodyFree(plat);
	cpSpaceRemoveShape(space, ground); cpShapeFree(ground);
	cpSpaceFree(space);
	return 0;
}
