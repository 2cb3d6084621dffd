/*
 * relink_program7.c -- an ordinary Chipmunk2D program (reference public API
 * only) built on the joints' own callbacks (cpConstraintSetPreSolveFunc,
 * cpConstraintSetPostSolveFunc; cpSpaceStep.c:389-396, 428-434): a chain
 * of pivot joints that break when their impulse passes a limit (post-solve
 * reads the impulse and queues the removal in a post-step callback), a
 * simple motor whose rate a pre-solve callback steers from the wheel's
 * angle, a damped spring whose rest length a pre-solve callback changes,
 * and a pin joint whose post-solve callback sums impulses.  The callbacks
 * check that the space is locked.  It prints the counters, the breaks,
 * the sums and every body's state.  Built like relink_program.c.
 */
#include <stdio.h>
#include <stdlib.h>
#ifdef RELINK_REFERENCE_HEADERS
#include "chipmunk/chipmunk.h"
#else
#include "chipmunk_gb300.h"
#endif

#define NLINK 12

static cpBody *links[NLINK];
static cpConstraint *joints[NLINK];
static int broken[NLINK];
static int nbroken, npre, npost, unlocked;
static cpFloat pinSum;
static cpBody *wheel;
static cpConstraint *spring;
static int stepNo;

static void remove_joint(cpSpace *space, void *key, void *data)
{
	(void)data;
	cpConstraint *j = (cpConstraint *)key;
	cpSpaceRemoveConstraint(space, j);
	printf("break %d %d\n", stepNo, (int)(size_t)cpConstraintGetUserData(j));
}

static void breakable_post(cpConstraint *j, cpSpace *space)
{
	npost++;
	if(!cpSpaceIsLocked(space)) unlocked++;
	cpFloat dt = cpSpaceGetCurrentTimeStep(space);
	cpFloat force = cpConstraintGetImpulse(j)/dt;
	int k = (int)(size_t)cpConstraintGetUserData(j);
	if(force > 2500.0 && !broken[k]){
		broken[k] = 1;
		nbroken++;
		cpSpaceAddPostStepCallback(space, remove_joint, j, NULL);
	}
}

static void motor_pre(cpConstraint *m, cpSpace *space)
{
	npre++;
	if(!cpSpaceIsLocked(space)) unlocked++;
	/* steer the wheel back towards angle 0 at most 3 rad/s */
	cpFloat a = cpBodyGetAngle(wheel);
	cpFloat rate = -2.0*a;
	if(rate > 3.0) rate = 3.0;
	if(rate < -3.0) rate = -3.0;
	cpSimpleMotorSetRate(m, rate);
}

static void spring_pre(cpConstraint *s, cpSpace *space)
{
	npre++;
	(void)space;
	cpDampedSpringSetRestLength(s, 30.0 + 10.0*((stepNo/40) % 2));
}

static void pin_post(cpConstraint *p, cpSpace *space)
{
	npost++;
	(void)space;
	pinSum += cpConstraintGetImpulse(p);
}

int main(void)
{
	cpSpace *space = cpSpaceNew();
	cpSpaceSetIterations(space, 12);
	cpSpaceSetGravity(space, cpv(0.0, -100.0));
	cpBody *sb = cpSpaceGetStaticBody(space);
	cpShape *ground = cpSpaceAddShape(space, cpSegmentShapeNew(sb, cpv(-300.0, -120.0), cpv(300.0, -120.0), 1.0));
	cpShapeSetFriction(ground, 1.0);

	/* a chain hanging from the static body, with a heavy weight at its end */
	cpBody *prev = sb;
	cpVect anchor = cpv(-100.0, 100.0);
	for(int i = 0; i < NLINK; i++){
		cpFloat m = (i == NLINK - 1) ? 6.0 : 0.5;
		cpBody *b = cpSpaceAddBody(space, cpBodyNew(m, cpMomentForBox(m, 8.0, 2.0)));
		cpBodySetPosition(b, cpv(-100.0 + 8.0*i + 4.0, 100.0));
		cpShape *s = cpSpaceAddShape(space, cpBoxShapeNew(b, 8.0, 2.0, 0.0));
		cpShapeSetFilter(s, cpShapeFilterNew(1, CP_ALL_CATEGORIES, CP_ALL_CATEGORIES));
		cpConstraint *j = cpSpaceAddConstraint(space, cpPivotJointNew(prev, b, anchor));
		cpConstraintSetUserData(j, (cpDataPointer)(size_t)i);
		cpConstraintSetPostSolveFunc(j, breakable_post);
		links[i] = b; joints[i] = j;
		prev = b;
		anchor = cpv(-100.0 + 8.0*(i + 1), 100.0);
	}

	/* a wheel on an axle, driven by a steered motor, with a ball on it */
	wheel = cpSpaceAddBody(space, cpBodyNew(2.0, cpMomentForCircle(2.0, 0.0, 15.0, cpvzero)));
	cpBodySetPosition(wheel, cpv(80.0, 0.0));
	cpBodySetAngle(wheel, 1.2);
	cpShape *ws = cpSpaceAddShape(space, cpCircleShapeNew(wheel, 15.0, cpvzero));
	cpShapeSetFriction(ws, 0.9);
	cpSpaceAddConstraint(space, cpPivotJointNew(sb, wheel, cpv(80.0, 0.0)));
	cpConstraint *motor = cpSpaceAddConstraint(space, cpSimpleMotorNew(sb, wheel, 0.0));
	cpConstraintSetMaxForce(motor, 4000.0);
	cpConstraintSetPreSolveFunc(motor, motor_pre);
	cpBody *ball = cpSpaceAddBody(space, cpBodyNew(0.5, cpMomentForCircle(0.5, 0.0, 4.0, cpvzero)));
	cpBodySetPosition(ball, cpv(82.0, 25.0));
	cpShape *bs = cpSpaceAddShape(space, cpCircleShapeNew(ball, 4.0, cpvzero));
	cpShapeSetFriction(bs, 0.7);

	/* a box on a spring whose rest length changes, pinned to a second box */
	cpBody *box = cpSpaceAddBody(space, cpBodyNew(1.0, cpMomentForBox(1.0, 10.0, 10.0)));
	cpBodySetPosition(box, cpv(160.0, 40.0));
	cpShape *xs = cpSpaceAddShape(space, cpBoxShapeNew(box, 10.0, 10.0, 0.0));
	cpShapeSetFriction(xs, 0.6);
	spring = cpSpaceAddConstraint(space, cpDampedSpringNew(sb, box, cpv(160.0, 80.0), cpvzero, 30.0, 60.0, 1.5));
	cpConstraintSetPreSolveFunc(spring, spring_pre);
	cpBody *box2 = cpSpaceAddBody(space, cpBodyNew(0.7, cpMomentForBox(0.7, 6.0, 6.0)));
	cpBodySetPosition(box2, cpv(175.0, 30.0));
	cpShape *xs2 = cpSpaceAddShape(space, cpBoxShapeNew(box2, 6.0, 6.0, 0.0));
	cpShapeSetFriction(xs2, 0.6);
	cpConstraint *pin = cpSpaceAddConstraint(space, cpPinJointNew(box, box2, cpv(5.0, 0.0), cpv(-3.0, 0.0)));
	cpConstraintSetPostSolveFunc(pin, pin_post);

	for(stepNo = 0; stepNo < 300; stepNo++){
		cpSpaceStep(space, 1.0/60.0);
		if(stepNo == 60){
			/* a kick that breaks the chain near the top */
			cpBodyApplyImpulseAtWorldPoint(links[NLINK - 1], cpv(0.0, -900.0), cpBodyGetPosition(links[NLINK - 1]));
		}
	}
	printf("counts %d %d %d %d\n", npre, npost, nbroken, unlocked);
	printf("pinsum %a\n", pinSum);
	for(int i = 0; i < NLINK; i++){
		cpVect p = cpBodyGetPosition(links[i]), v = cpBodyGetVelocity(links[i]);
		printf("%d %a %a %a %a %a %a\n", i, p.x, p.y, v.x, v.y, cpBodyGetAngle(links[i]), cpBodyGetAngularVelocity(links[i]));
	}
	cpBody *others[4] = { wheel, ball, box, box2 };
	for(int i = 0; i < 4; i++){
		cpVect p = cpBodyGetPosition(others[i]), v = cpBodyGetVelocity(others[i]);
		printf("%d %a %a %a %a %a %a\n", 100 + i, p.x, p.y, v.x, v.y, cpBodyGetAngle(others[i]), cpBodyGetAngularVelocity(others[i]));
	}
	printf("motor %a\n", cpSimpleMotorGetRate(motor));
	cpSpaceFree(space);
	return 0;
}
