/*
 * relink_program2.c -- an ordinary Chipmunk2D program (reference public API
 * only) that places its objects in memory it asks the library for
 * (cp*Alloc / cp*Init / cp*Destroy), uses the threaded space's entry
 * points (cpHastySpace.h), every joint kind, the space queries, a
 * post-step callback that removes a body, and the shape iteration order,
 * then prints every body's state and the queries' results as hexadecimal
 * floats.  Built like relink_program.c.
 */
#include <stdio.h>
#include <stdlib.h>
#ifdef RELINK_REFERENCE_HEADERS
#include "chipmunk/chipmunk.h"
#include "chipmunk/cpHastySpace.h"
#else
#include "chipmunk_gb300.h"
#endif

#define NB 24

static cpBody *bodies[NB];
static cpShape *shapes[NB];

/* a post-step callback that takes a body and its shape out of the space */
static void remove_later(cpSpace *space, void *key, void *data)
{
	int i = (int)(size_t)data;
	(void)key;
	cpSpaceRemoveShape(space, shapes[i]); cpShapeDestroy(shapes[i]); free(shapes[i]);
	cpSpaceRemoveBody(space, bodies[i]); cpBodyDestroy(bodies[i]); free(bodies[i]);
	bodies[i] = NULL; shapes[i] = NULL;
}

static void print_shape(cpShape *shape, void *data)
{
	(void)data;
	printf(" %d", (int)(size_t)cpShapeGetUserData(shape));
}

static void print_nearest(cpSpace *space, cpVect p)
{
	cpPointQueryInfo info;
	cpShape *s = cpSpacePointQueryNearest(space, p, 50.0, CP_SHAPE_FILTER_ALL, &info);
	printf("nearest %d %a %a %a %a %a\n", s != NULL, info.point.x, info.point.y, info.distance, info.gradient.x, info.gradient.y);
}

static void print_ray(cpSpace *space, cpVect a, cpVect b)
{
	cpSegmentQueryInfo info;
	cpShape *s = cpSpaceSegmentQueryFirst(space, a, b, 0.5, CP_SHAPE_FILTER_ALL, &info);
	printf("ray %d %a %a %a %a %a\n", s != NULL, info.point.x, info.point.y, info.normal.x, info.normal.y, info.alpha);
}

int main(void)
{
	cpSpace *space = cpHastySpaceNew();
	/* one thread: the reference's threaded solver is deterministic only then */
	cpHastySpaceSetThreads(space, 1);
	cpSpaceSetGravity(space, cpv(0.0, -100.0));
	cpSpaceSetIterations(space, 12);

	cpShape *ground = (cpShape *)cpSegmentShapeInit(cpSegmentShapeAlloc(), cpSpaceGetStaticBody(space), cpv(-400.0, 0.0), cpv(400.0, 0.0), 1.0);
	cpShapeSetFriction(ground, 1.0);
	cpSpaceAddShape(space, ground);

	for(int i = 0; i < NB; i++){
		cpBody *b = cpBodyInit(cpBodyAlloc(), 1.0 + 0.1*i, 1.0);
		cpShape *s;
		if(i % 3 == 0){
			s = (cpShape *)cpCircleShapeInit(cpCircleShapeAlloc(), b, 4.0 + (i % 4), cpvzero);
			cpBodySetMoment(b, cpMomentForCircle(cpBodyGetMass(b), 0.0, 4.0 + (i % 4), cpvzero));
		} else if(i % 3 == 1){
			s = (cpShape *)cpBoxShapeInit(cpPolyShapeAlloc(), b, 10.0, 6.0, 0.5);
			cpBodySetMoment(b, cpMomentForBox(cpBodyGetMass(b), 10.0, 6.0));
		} else {
			cpVect verts[5] = { cpv(-5.0, -3.0), cpv(5.0, -4.0), cpv(6.0, 2.0), cpv(0.0, 6.0), cpv(-6.0, 3.0) };
			s = (cpShape *)cpPolyShapeInit(cpPolyShapeAlloc(), b, 5, verts, cpTransformIdentity, 0.0);
			cpBodySetMoment(b, cpMomentForPoly(cpBodyGetMass(b), 5, verts, cpvzero, 0.0));
		}
		cpBodySetPosition(b, cpv(-120.0 + 22.0*(i % 12), 20.0 + 30.0*(i/12)));
		cpShapeSetFriction(s, 0.6);
		cpShapeSetUserData(s, (cpDataPointer)(size_t)(i + 1));
		cpSpaceAddBody(space, b);
		cpSpaceAddShape(space, s);
		bodies[i] = b; shapes[i] = s;
	}
	cpConstraint *joints[10];
	joints[0] = (cpConstraint *)cpPivotJointInit(cpPivotJointAlloc(), bodies[0], bodies[1], cpvzero, cpv(0.0, 5.0));
	joints[1] = (cpConstraint *)cpPinJointInit(cpPinJointAlloc(), bodies[2], bodies[3], cpvzero, cpvzero);
	joints[2] = (cpConstraint *)cpSlideJointInit(cpSlideJointAlloc(), bodies[4], bodies[5], cpvzero, cpvzero, 10.0, 30.0);
	joints[3] = (cpConstraint *)cpGrooveJointInit(cpGrooveJointAlloc(), bodies[6], bodies[7], cpv(-10.0, 0.0), cpv(10.0, 0.0), cpvzero);
	joints[4] = (cpConstraint *)cpDampedSpringInit(cpDampedSpringAlloc(), bodies[8], bodies[9], cpvzero, cpvzero, 20.0, 50.0, 2.0);
	joints[5] = (cpConstraint *)cpDampedRotarySpringInit(cpDampedRotarySpringAlloc(), bodies[10], bodies[11], 0.5, 300.0, 10.0);
	joints[6] = (cpConstraint *)cpRotaryLimitJointInit(cpRotaryLimitJointAlloc(), bodies[12], bodies[13], -0.3, 0.3);
	joints[7] = (cpConstraint *)cpRatchetJointInit(cpRatchetJointAlloc(), bodies[14], bodies[15], 0.0, 0.4);
	joints[8] = (cpConstraint *)cpGearJointInit(cpGearJointAlloc(), bodies[16], bodies[17], 0.0, 2.0);
	joints[9] = (cpConstraint *)cpSimpleMotorInit(cpSimpleMotorAlloc(), bodies[18], bodies[19], 1.5);
	for(int k = 0; k < 10; k++) cpSpaceAddConstraint(space, joints[k]);

	for(int step = 0; step < 150; step++){
		cpHastySpaceStep(space, 1.0/60.0);
		if(step == 75){
			print_nearest(space, cpv(-100.0, 10.0));
			print_ray(space, cpv(-200.0, 15.0), cpv(200.0, 15.0));
		}
		if(step == 100){
			/* runs when the next step ends; a second callback on the same key is refused */
			cpBool first = cpSpaceAddPostStepCallback(space, remove_later, bodies + 21, (void *)(size_t)21);
			cpBool again = cpSpaceAddPostStepCallback(space, remove_later, bodies + 21, (void *)(size_t)21);
			printf("poststep %d %d\n", (int)first, (int)again);
		}
	}
	printf("order");
	cpSpaceEachShape(space, print_shape, NULL);
	printf("\n");
	printf("threads %lu\n", cpHastySpaceGetThreads(space) > 0 ? 1ul : 0ul);
	for(int i = 0; i < NB; i++){
		if(!bodies[i]) continue;
		cpVect p = cpBodyGetPosition(bodies[i]), v = cpBodyGetVelocity(bodies[i]);
		printf("%d %a %a %a %a %a %a\n", i, p.x, p.y, v.x, v.y, cpBodyGetAngle(bodies[i]), cpBodyGetAngularVelocity(bodies[i]));
	}
	print_nearest(space, cpv(0.0, 5.0));
	print_ray(space, cpv(-200.0, 4.0), cpv(200.0, 8.0));

	for(int k = 0; k < 10; k++){ cpSpaceRemoveConstraint(space, joints[k]); cpConstraintDestroy(joints[k]); free(joints[k]); }
	for(int i = 0; i < NB; i++){
		if(!bodies[i]) continue;
		cpSpaceRemoveShape(space, shapes[i]); cpShapeDestroy(shapes[i]); free(shapes[i]);
		cpSpaceRemoveBody(space, bodies[i]); cpBodyDestroy(bodies[i]); free(bodies[i]);
	}
	cpSpaceRemoveShape(space, ground); cpShapeDestroy(ground); free(ground);
	cpHastySpaceFree(space);
	return 0;
}
