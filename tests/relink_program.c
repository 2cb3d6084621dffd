/*
 * relink_program.c -- an ordinary Chipmunk2D program, written against the
 * reference's public C API only.  It builds a stack of boxes, balls and
 * joints, steps it, removes and frees bodies, shapes and a joint, adds
 * new ones and another joint mid-run, and prints every body's state as
 * hexadecimal floats.  The tests build it unchanged against either the
 * reference's headers (RELINK_REFERENCE_HEADERS, include path to its
 * include/) or this repository's header, and link it against each
 * implementation of the API.
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

static void add_box(cpSpace *space, cpVect p, cpFloat w, cpFloat h)
{
	cpBody *b = cpSpaceAddBody(space, cpBodyNew(1.0, cpMomentForBox(1.0, w, h)));
	cpBodySetPosition(b, p);
	cpShape *s = cpSpaceAddShape(space, cpBoxShapeNew(b, w, h, 0.0));
	cpShapeSetFriction(s, 0.7);
	bodies[nbodies] = b; shapes[nbodies] = s; nbodies++;
}

static void add_ball(cpSpace *space, cpVect p, cpFloat r, cpVect v)
{
	cpBody *b = cpSpaceAddBody(space, cpBodyNew(2.0, cpMomentForCircle(2.0, 0.0, r, cpvzero)));
	cpBodySetPosition(b, p);
	cpBodySetVelocity(b, v);
	cpShape *s = cpSpaceAddShape(space, cpCircleShapeNew(b, r, cpvzero));
	cpShapeSetFriction(s, 0.5);
	cpShapeSetElasticity(s, 0.2);
	bodies[nbodies] = b; shapes[nbodies] = s; nbodies++;
}

static void remove_body(cpSpace *space, int i)
{
	cpSpaceRemoveShape(space, shapes[i]);
	cpSpaceRemoveBody(space, bodies[i]);
	cpShapeFree(shapes[i]);
	cpBodyFree(bodies[i]);
	bodies[i] = NULL; shapes[i] = NULL;
}

int main(void)
{
	cpSpace *space = cpSpaceNew();
	cpSpaceSetIterations(space, 10);
	cpSpaceSetGravity(space, cpv(0.0, -100.0));
	cpShape *ground = cpSpaceAddShape(space, cpSegmentShapeNew(cpSpaceGetStaticBody(space), cpv(-320.0, 0.0), cpv(320.0, 0.0), 0.0));
	cpShapeSetFriction(ground, 1.0);
	for(int i = 0; i < 6; i++)
		for(int j = 0; j < 5; j++) add_box(space, cpv(-60.0 + 24.0*j + 3.0*(i & 1), 6.0 + 12.0*i), 10.0, 10.0);
	for(int k = 0; k < 4; k++) add_ball(space, cpv(-90.0 + 60.0*k, 120.0 + 7.0*k), 3.0 + k, cpv(10.0 - 5.0*k, 0.0));
	cpConstraint *pivot = cpSpaceAddConstraint(space, cpPivotJointNew(bodies[25], bodies[26], cpvlerp(cpBodyGetPosition(bodies[25]), cpBodyGetPosition(bodies[26]), 0.5)));
	cpConstraint *pin = cpSpaceAddConstraint(space, cpPinJointNew(bodies[30], bodies[31], cpvzero, cpvzero));
	cpConstraint *slide = NULL;
	for(int step = 0; step < 180; step++){
		cpSpaceStep(space, 1.0/60.0);
		if(step == 40){
			/* three boxes off the top of the stack */
			remove_body(space, 27);
			remove_body(space, 28);
			remove_body(space, 29);
		}
		if(step == 70){
			for(int k = 0; k < 5; k++) add_ball(space, cpv(-40.0 + 20.0*k, 140.0), 2.5, cpv(0.0, -20.0));
		}
		if(step == 100){
			cpSpaceRemoveConstraint(space, pivot);
			cpConstraintFree(pivot);
			pivot = NULL;
			slide = cpSpaceAddConstraint(space, cpSlideJointNew(bodies[34], bodies[35], cpvzero, cpvzero, 5.0, 40.0));
			cpPinJointSetDist(pin, cpPinJointGetDist(pin)*0.9);
		}
		if(step == 130){
			remove_body(space, 2);
			add_box(space, cpv(100.0, 30.0), 14.0, 8.0);
		}
	}
	for(int i = 0; i < nbodies; i++){
		if(!bodies[i]) continue;
		cpVect p = cpBodyGetPosition(bodies[i]), v = cpBodyGetVelocity(bodies[i]);
		printf("%d %a %a %a %a %a %a\n", i, p.x, p.y, v.x, v.y, cpBodyGetAngle(bodies[i]), cpBodyGetAngularVelocity(bodies[i]));
	}
	if(slide){ cpSpaceRemoveConstraint(space, slide); cpConstraintFree(slide); }
	cpSpaceRemoveConstraint(space, pin); cpConstraintFree(pin);
	for(int i = 0; i < nbodies; i++) if(bodies[i]) remove_body(space, i);
	cpSpaceRemoveShape(space, ground);
	cpShapeFree(ground);
	cpSpaceFree(space);
	return 0;
}
