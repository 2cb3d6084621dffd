/*
 * relink_program8.c -- an ordinary Chipmunk2D program (reference public API
 * only) with bodies that carry their own velocity function
 * (cpBodySetVelocityUpdateFunc; cpSpaceStep.c:399-403): boxes and balls
 * pulled towards a static planet by an inverse-square field computed from
 * their own position and handed to cpBodyUpdateVelocity, one body whose
 * function adds its own drag and keeps the forces applied to it, bodies
 * with the default update beside them, and a pivot joint between a custom
 * body and a default one.  It prints every body's state.  Built like
 * relink_program.c.
 */
#include <stdio.h>
#include <stdlib.h>
#include <math.h>
#ifdef RELINK_REFERENCE_HEADERS
#include "chipmunk/chipmunk.h"
#else
#include "chipmunk_gb300.h"
#endif

#define NB 24

static cpBody *bodies[NB];
static int calls;

static void planet_gravity(cpBody *body, cpVect gravity, cpFloat damping, cpFloat dt)
{
	(void)gravity;
	calls++;
	cpVect p = cpBodyGetPosition(body);
	cpFloat sq = cpvlengthsq(p);
	cpVect g = cpvmult(p, -5.0e6/(sq*sqrt(sq)));
	cpBodyUpdateVelocity(body, g, damping, dt);
}

static void own_drag(cpBody *body, cpVect gravity, cpFloat damping, cpFloat dt)
{
	(void)damping;
	calls++;
	cpVect v = cpBodyGetVelocity(body);
	cpBodySetVelocity(body, cpvadd(cpvmult(v, 0.98), cpvmult(gravity, dt)));
	cpBodySetAngularVelocity(body, cpBodyGetAngularVelocity(body)*0.95);
}

int main(void)
{
	cpSpace *space = cpSpaceNew();
	cpSpaceSetIterations(space, 10);
	cpSpaceSetGravity(space, cpv(0.0, -30.0));
	cpSpaceSetDamping(space, 0.9);
	cpBody *planet = cpSpaceAddBody(space, cpBodyNewKinematic());
	cpBodySetAngularVelocity(planet, 0.2);
	cpShape *ps = cpSpaceAddShape(space, cpCircleShapeNew(planet, 70.0, cpvzero));
	cpShapeSetFriction(ps, 1.0);
	for(int i = 0; i < NB; i++){
		cpFloat ang = 2.0*M_PI*i/NB, r = 120.0 + 9.0*(i % 4);
		cpBody *b;
		cpShape *s;
		if(i % 2){
			b = cpBodyNew(1.0, cpMomentForBox(1.0, 8.0, 6.0));
			s = cpBoxShapeNew(b, 8.0, 6.0, 0.0);
		} else {
			b = cpBodyNew(0.8, cpMomentForCircle(0.8, 0.0, 4.0, cpvzero));
			s = cpCircleShapeNew(b, 4.0, cpvzero);
		}
		cpBodySetPosition(b, cpv(r*cos(ang), r*sin(ang)));
		cpBodySetVelocity(b, cpv(-40.0*sin(ang), 40.0*cos(ang)));
		cpSpaceAddBody(space, b);
		cpSpaceAddShape(space, s);
		cpShapeSetFriction(s, 0.7);
		if(i % 6 != 5) cpBodySetVelocityUpdateFunc(b, planet_gravity);
		bodies[i] = b;
	}
	cpBodySetVelocityUpdateFunc(bodies[5], own_drag);
	cpSpaceAddConstraint(space, cpPivotJointNew(bodies[0], bodies[1], cpvlerp(cpBodyGetPosition(bodies[0]), cpBodyGetPosition(bodies[1]), 0.5)));
	for(int step = 0; step < 240; step++){
		if(step % 30 == 0) cpBodyApplyForceAtLocalPoint(bodies[5], cpv(50.0, 0.0), cpvzero);
		cpSpaceStep(space, 1.0/60.0);
	}
	printf("calls %d\n", calls);
	for(int i = 0; i < NB; i++){
		cpVect p = cpBodyGetPosition(bodies[i]), v = cpBodyGetVelocity(bodies[i]), f = cpBodyGetForce(bodies[i]);
		printf("%d %a %a %a %a %a %a %a %a\n", i, p.x, p.y, v.x, v.y, cpBodyGetAngle(bodies[i]), cpBodyGetAngularVelocity(bodies[i]), f.x, f.y);
	}
	return 0;
}
