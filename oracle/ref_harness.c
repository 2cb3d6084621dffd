/*
 * ref_harness.c -- state export for the unmodified Chipmunk2D reference.
 *
 * Test infrastructure.  Compiled only by oracle/build_ref.sh, together with
 * the reference sources from their read-only location, into
 * oracle/_ref/libcpref.so.  It reads the reference's private structs
 * (include/chipmunk/chipmunk_structs.h:35-305) and writes them in the fixed
 * record layouts shared by every implementation in this repository:
 *   bodies      18 doubles per dynamic body (space->dynamicBodies order)
 *   arbiters    34 doubles per arbiter (space->arbiters order = solve order)
 *   constraints  8 doubles per constraint (space->constraints order)
 */
#include <string.h>
#include "chipmunk/chipmunk_private.h"
#include "chipmunk/cpHastySpace.h"

/* cpConstraintClass pointers identify the joint kind. */
#define KIND_PIVOT 1.0
#define KIND_PIN 2.0
#define KIND_SLIDE 3.0

int cpx_dump_bodies(cpSpace *space, double *out, int max)
{
	cpArray *bodies = space->dynamicBodies;
	for(int i = 0; i < bodies->num && i < max; i++){
		cpBody *b = (cpBody *)bodies->arr[i];
		double *o = out + 18*i;
		o[0] = b->p.x; o[1] = b->p.y; o[2] = b->v.x; o[3] = b->v.y; o[4] = b->a; o[5] = b->w;
		o[6] = b->f.x; o[7] = b->f.y; o[8] = b->t; o[9] = b->v_bias.x; o[10] = b->v_bias.y; o[11] = b->w_bias;
		o[12] = b->transform.a; o[13] = b->transform.b; o[14] = b->transform.c; o[15] = b->transform.d;
		o[16] = b->transform.tx; o[17] = b->transform.ty;
	}
	return bodies->num;
}

int cpx_set_bodies(cpSpace *space, const double *in, int count)
{
	cpArray *bodies = space->dynamicBodies;
	for(int i = 0; i < bodies->num && i < count; i++){
		cpBody *b = (cpBody *)bodies->arr[i];
		const double *o = in + 18*i;
		b->p.x = o[0]; b->p.y = o[1]; b->v.x = o[2]; b->v.y = o[3]; b->a = o[4]; b->w = o[5];
		b->f.x = o[6]; b->f.y = o[7]; b->t = o[8]; b->v_bias.x = o[9]; b->v_bias.y = o[10]; b->w_bias = o[11];
		b->transform.a = o[12]; b->transform.b = o[13]; b->transform.c = o[14]; b->transform.d = o[15];
		b->transform.tx = o[16]; b->transform.ty = o[17];
	}
	return bodies->num;
}

int cpx_dump_arbiters(cpSpace *space, double *out, int max)
{
	cpArray *arbiters = space->arbiters;
	for(int i = 0; i < arbiters->num && i < max; i++){
		cpArbiter *arb = (cpArbiter *)arbiters->arr[i];
		double *o = out + 34*i;
		memset(o, 0, 34*sizeof(double));
		o[0] = (double)arb->a->hashid; o[1] = (double)arb->b->hashid; o[2] = arb->count; o[3] = arb->state;
		o[4] = arb->n.x; o[5] = arb->n.y; o[6] = arb->e; o[7] = arb->u; o[8] = arb->surface_vr.x; o[9] = arb->surface_vr.y;
		for(int c = 0; c < arb->count; c++){
			struct cpContact *con = &arb->contacts[c];
			double *q = o + 10 + 12*c;
			q[0] = con->r1.x; q[1] = con->r1.y; q[2] = con->r2.x; q[3] = con->r2.y;
			q[4] = con->nMass; q[5] = con->tMass; q[6] = con->bounce; q[7] = con->jnAcc; q[8] = con->jtAcc;
			q[9] = con->jBias; q[10] = con->bias; q[11] = (double)(con->hash & 0xffffffffffffULL);
		}
	}
	return arbiters->num;
}

int cpx_dump_constraints(cpSpace *space, double *out, int max)
{
	cpArray *constraints = space->constraints;
	for(int i = 0; i < constraints->num && i < max; i++){
		cpConstraint *c = (cpConstraint *)constraints->arr[i];
		double *o = out + 8*i;
		memset(o, 0, 8*sizeof(double));
		if(cpConstraintIsPivotJoint(c)){
			cpPivotJoint *j = (cpPivotJoint *)c;
			o[0] = KIND_PIVOT; o[1] = j->jAcc.x; o[2] = j->jAcc.y;
			o[3] = j->r1.x; o[4] = j->r1.y; o[5] = j->r2.x; o[6] = j->r2.y; o[7] = j->bias.x;
		} else if(cpConstraintIsPinJoint(c)){
			cpPinJoint *j = (cpPinJoint *)c;
			o[0] = KIND_PIN; o[1] = j->jnAcc; o[2] = j->nMass;
			o[3] = j->r1.x; o[4] = j->r1.y; o[5] = j->r2.x; o[6] = j->r2.y; o[7] = j->bias;
		} else if(cpConstraintIsSlideJoint(c)){
			cpSlideJoint *j = (cpSlideJoint *)c;
			o[0] = KIND_SLIDE; o[1] = j->jnAcc; o[2] = j->nMass;
			o[3] = j->r1.x; o[4] = j->r1.y; o[5] = j->r2.x; o[6] = j->r2.y; o[7] = j->bias;
		} else if(cpConstraintIsGrooveJoint(c)){
			cpGrooveJoint *j = (cpGrooveJoint *)c;
			o[0] = 4; o[1] = j->jAcc.x; o[2] = j->jAcc.y;
			o[3] = j->r1.x; o[4] = j->r1.y; o[5] = j->r2.x; o[6] = j->r2.y; o[7] = j->bias.x;
		} else if(cpConstraintIsDampedSpring(c)){
			cpDampedSpring *j = (cpDampedSpring *)c;
			o[0] = 5; o[1] = j->jAcc; o[2] = j->nMass;
			o[3] = j->r1.x; o[4] = j->r1.y; o[5] = j->r2.x; o[6] = j->r2.y; o[7] = j->v_coef;
		} else if(cpConstraintIsDampedRotarySpring(c)){
			cpDampedRotarySpring *j = (cpDampedRotarySpring *)c;
			o[0] = 6; o[1] = j->jAcc; o[2] = j->iSum; o[3] = j->w_coef; o[7] = j->target_wrn;
		} else if(cpConstraintIsRotaryLimitJoint(c)){
			cpRotaryLimitJoint *j = (cpRotaryLimitJoint *)c;
			o[0] = 7; o[1] = j->jAcc; o[2] = j->iSum; o[7] = j->bias;
		} else if(cpConstraintIsRatchetJoint(c)){
			cpRatchetJoint *j = (cpRatchetJoint *)c;
			o[0] = 8; o[1] = j->jAcc; o[2] = j->iSum; o[3] = j->angle; o[7] = j->bias;
		} else if(cpConstraintIsGearJoint(c)){
			cpGearJoint *j = (cpGearJoint *)c;
			o[0] = 9; o[1] = j->jAcc; o[2] = j->iSum; o[7] = j->bias;
		} else if(cpConstraintIsSimpleMotor(c)){
			cpSimpleMotor *j = (cpSimpleMotor *)c;
			o[0] = 10; o[1] = j->jAcc; o[2] = j->iSum;
		}
	}
	return constraints->num;
}

/* Threaded reference solver (cpHastySpace) for the CPU baseline. */
cpSpace *cpx_hasty_new(int threads)
{
	cpSpace *space = cpHastySpaceNew();
	cpHastySpaceSetThreads(space, (unsigned long)threads);
	return space;
}

void cpx_hasty_step(cpSpace *space, double dt) { cpHastySpaceStep(space, dt); }
