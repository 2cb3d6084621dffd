/*
 * relink_program9.c -- an ordinary Chipmunk2D program (reference public API
 * only) with bodies that carry their own position function
 * (cpBodySetPositionUpdateFunc; cpSpaceStep.c:362-366): balls whose
 * function runs cpBodyUpdatePosition and then keeps them inside a wall by
 * reflecting position and velocity, a box whose function rotates it at a
 * fixed rate, and default bodies on a ground segment beside them.  It
 * prints every body's state.  Built like relink_program.c.
 */
#include <stdio.h>
#include <stdlib.h>
#ifdef RELINK_REFERENCE_HEADERS
#include "chipmunk/chipmunk.h"
#else
#include "chipmunk_gb300.h"
#endif

#define NB 20

static cpBody *bodies[NB];
static int calls;

static void walled(cpBody *body, cpFloat dt)
{
	calls++;
	cpBodyUpdatePosition(body, dt);
	cpVect p = cpBodyGetPosition(body), v = cpBodyGetVelocity(body);
	if(p.x > 60.0){
		cpBodySetPosition(body, cpv(120.0 - p.x, p.y));
		cpBodySetVelocity(body, cpv(-v.x, v.y));
	}
}

static void spinner(cpBody *body, cpFloat dt)
{
	calls++;
	cpBodySetAngularVelocity(body, 1.5);
	cpBodyUpdatePosition(body, dt);
}

int main(void)
{
	cpSpace *space = cpSpaceNew();
	cpSpaceSetIterations(space, 10);
	cpSpaceSetGravity(space, cpv(0.0, -100.0));
	cpShape *ground = cpSpaceAddShape(space, cpSegmentShapeNew(cpSpaceGetStaticBody(space), cpv(-200.0, 0.0), cpv(200.0, 0.0), 1.0));
	cpShapeSetFriction(ground, 1.0);
	cpShapeSetElasticity(ground, 0.5);
	for(int i = 0; i < NB; i++){
		cpBody *b;
		cpShape *s;
		if(i % 3 == 2){
			b = cpBodyNew(1.0, cpMomentForBox(1.0, 10.0, 6.0));
			s = cpBoxShapeNew(b, 10.0, 6.0, 0.0);
		} else {
			b = cpBodyNew(0.6, cpMomentForCircle(0.6, 0.0, 3.5, cpvzero));
			s = cpCircleShapeNew(b, 3.5, cpvzero);
		}
		cpBodySetPosition(b, cpv(-50.0 + 9.0*i, 20.0 + 7.0*(i % 5)));
		cpBodySetVelocity(b, cpv(30.0 + 4.0*i, 0.0));
		cpSpaceAddBody(space, b);
		cpSpaceAddShape(space, s);
		cpShapeSetFriction(s, 0.6);
		cpShapeSetElasticity(s, 0.5);
		if(i % 3 == 0) cpBodySetPositionUpdateFunc(b, walled);
		bodies[i] = b;
	}
	cpBodySetPositionUpdateFunc(bodies[5], spinner);
	for(int step = 0; step < 240; step++) cpSpaceStep(space, 1.0/60.0);
	printf("calls %d\n", calls);
	for(int i = 0; i < NB; i++){
		cpVect p = cpBodyGetPosition(bodies[i]), v = cpBodyGetVelocity(bodies[i]);
		printf("%d %a %a %a %a %a %a\n", i, p.x, p.y, v.x, v.y, cpBodyGetAngle(bodies[i]), cpBodyGetAngularVelocity(bodies[i]));
	}
	return 0;
}
