/*
 * cpg_adjoint.cuh -- reverse-mode derivatives of one step of the
 * reference-order step, for the differentiable rollout.
 *
 * Everything here is plain arithmetic on doubles, usable on the device and
 * on the host (the host build checks it against finite differences).  The
 * forward quantities are recomputed from taped values with the forward's
 * own expressions, so every branch (max/clamp activity, clamp side, region
 * of a closest point, contact push) is taken exactly as in the forward.
 *
 * Pieces, in the order the forward runs them (cpSpaceStep.c:335-445):
 *  - contact geometry (cpCollision.c): the contact points p1, p2 and the
 *    normal n of a pair as functions of the poses (position, angle) of its
 *    two bodies, evaluated in 6-component dual numbers from the forward's
 *    world geometry and final GJK/EPA features (geom_*);
 *  - arbiter pre-step (cpArbiter.c:416-439): nMass, tMass, bias, bounce
 *    (prestep_adjoint);
 *  - warm start (cpArbiter.c:441-455) and one impulse application
 *    (cpArbiter.c:459-498) (warm_adjoint, app_adjoint).
 * Integration (cpBody.c:493-522) is linear in the carried state and is
 * handled by the kernels directly.
 */
#pragma once
#include <cfloat>
#include <cmath>
#include <cstring>

#ifdef __CUDACC__
#define CPG_HD __host__ __device__ __forceinline__
#else
#define CPG_HD inline
#endif

/* ---------------------------------------------------------------------
 * Taped data of one application of one contact (one iteration).
 * ------------------------------------------------------------------- */
struct AdjApp {
	double jN0, jT0, jB0;        /* accumulators before: jnAcc, jtAcc, jBias */
	double jN1, jT1, jB1;        /* after */
	double vrx, vry;             /* v2 - v1 + surface_vr at the contact */
	double vbx, vby;             /* vb2 - vb1 */
	double wA, wB, wbA, wbB;     /* angular (bias) velocities before */
};

/* Constants of a contact during the solve. */
struct AdjCon {
	double r1x, r1y, r2x, r2y, nx, ny;
	double nMass, tMass, bias, bounce, u;
	double minvA, minvB, iinvA, iinvB;
};

/* Adjoints accumulated for a contact's constants. */
struct AdjConBar {
	double r1x, r1y, r2x, r2y, nx, ny;
	double nMass, tMass, bias, bounce, u;
	double minvA, minvB;
};

/* Adjoint of a body's velocity state. */
struct AdjBody { double vx, vy, w, vbx, vby, wb; };

CPG_HD void adj_zero(AdjConBar &c)
{
	c.r1x = c.r1y = c.r2x = c.r2y = c.nx = c.ny = 0.0;
	c.nMass = c.tMass = c.bias = c.bounce = c.u = 0.0;
	c.minvA = c.minvB = 0.0;
}

/* Adjoint of applying impulse J to A (as -J at r1) and B (at r2):
 *   vA' = vA + (-J)*minvA,  wA' = wA + iinvA*(r1 x (-J)),
 *   vB' = vB + J*minvB,     wB' = wB + iinvB*(r2 x J).
 * A, B hold the adjoints of the velocities after; they are the adjoints of
 * the velocities before as well (the map is the identity in them), so only
 * the adjoint of J and of r1, r2, minv are produced.  `bias` selects the
 * bias velocities. */
CPG_HD void adj_apply_pair(const AdjCon &c, double Jx, double Jy, const AdjBody &A, const AdjBody &B, bool bias,
	double &Jbx, double &Jby, AdjConBar &cb)
{
	double avx = bias ? A.vbx : A.vx, avy = bias ? A.vby : A.vy, aw = bias ? A.wb : A.w;
	double bvx = bias ? B.vbx : B.vx, bvy = bias ? B.vby : B.vy, bw = bias ? B.wb : B.w;
	Jbx = -c.minvA*avx + c.minvB*bvx;
	Jby = -c.minvA*avy + c.minvB*bvy;
	cb.minvA += -(Jx*avx + Jy*avy);
	cb.minvB += Jx*bvx + Jy*bvy;
	/* wA' = wA - iinvA*(r1.x*Jy - r1.y*Jx) */
	double gA = -c.iinvA*aw;
	cb.r1x += gA*Jy; cb.r1y += -gA*Jx;
	Jbx += -gA*c.r1y; Jby += gA*c.r1x;
	double gB = c.iinvB*bw;
	cb.r2x += gB*Jy; cb.r2y += -gB*Jx;
	Jbx += -gB*c.r2y; Jby += gB*c.r2x;
}

/* Adjoint of a relative velocity d = (vB + perp(r2)*wB) - (vA + perp(r1)*wA)
 * (perp(r)*w = (-r.y*w, r.x*w)) with adjoint (dbx, dby): adds into the
 * body adjoints (velocity or bias part) and r1, r2. */
CPG_HD void adj_relvel(const AdjCon &c, double dbx, double dby, double wA, double wB, AdjBody &A, AdjBody &B, bool bias, AdjConBar &cb)
{
	double dwA = dbx*c.r1y - dby*c.r1x;
	double dwB = -dbx*c.r2y + dby*c.r2x;
	if(bias){
		A.vbx -= dbx; A.vby -= dby; B.vbx += dbx; B.vby += dby;
		A.wb += dwA; B.wb += dwB;
	} else {
		A.vx -= dbx; A.vy -= dby; B.vx += dbx; B.vy += dby;
		A.w += dwA; B.w += dwB;
	}
	cb.r1y += dbx*wA; cb.r1x += -dby*wA;
	cb.r2y += -dbx*wB; cb.r2x += dby*wB;
}

/* Reverse of one application of one contact (cpArbiter.c:459-498).
 * On entry A, B are the adjoints of the bodies' velocity states after the
 * application and jNbar, jTbar, jBbar those of the accumulators after; on
 * return they are the adjoints before.  cb accumulates the adjoints of the
 * contact's constants. */
CPG_HD void app_adjoint(const AdjCon &c, const AdjApp &t, AdjBody &A, AdjBody &B,
	double &jNbar, double &jTbar, double &jBbar, AdjConBar &cb)
{
	double nx = c.nx, ny = c.ny;
	/* forward intermediates, with the forward's expressions */
	double vrn = t.vrx*nx + t.vry*ny;
	double vrt = t.vrx*(-ny) + t.vry*nx;
	double vbn = t.vbx*nx + t.vby*ny;
	double jbn = (c.bias - vbn)*c.nMass;
	bool activeB = (t.jB0 + jbn > 0.0);
	double jn = -(c.bounce + vrn)*c.nMass;
	bool activeN = (t.jN0 + jn > 0.0);
	double jtMax = c.u*t.jN1;
	double jt = -vrt*c.tMass;
	double f = t.jT0 + jt;
	/* dclamp(f, -jtMax, jtMax) = dmin(dmax(f, -jtMax), jtMax) */
	int side = (f > -jtMax) ? 0 : 1;            /* 0: f, 1: -jtMax */
	double m = side ? -jtMax : f;
	if(!(m < jtMax)) side = 2;                  /* 2: +jtMax */
	double dN = t.jN1 - t.jN0, dT = t.jT1 - t.jT0, db = t.jB1 - t.jB0;
	double Jx = nx*dN - ny*dT, Jy = nx*dT + ny*dN;
	double bx = nx*db, by = ny*db;

	/* ---- normal and friction impulse (velocities) ---- */
	double Jbx, Jby;
	adj_apply_pair(c, Jx, Jy, A, B, false, Jbx, Jby, cb);
	double dNbar = Jbx*nx + Jby*ny;
	double dTbar = -Jbx*ny + Jby*nx;
	cb.nx += Jbx*dN + Jby*dT;
	cb.ny += -Jbx*dT + Jby*dN;
	double jN1bar = jNbar + dNbar, jN0bar = -dNbar;
	double jT1bar = jTbar + dTbar, jT0bar = -dTbar;
	double fbar = 0.0, jtMaxbar = 0.0;
	if(side == 0) fbar = jT1bar; else if(side == 1) jtMaxbar = -jT1bar; else jtMaxbar = jT1bar;
	jT0bar += fbar;
	double vrtbar = -fbar*c.tMass;
	cb.tMass += -fbar*vrt;
	cb.u += jtMaxbar*t.jN1;
	jN1bar += jtMaxbar*c.u;
	double jnbar = 0.0;
	if(activeN){ jN0bar += jN1bar; jnbar = jN1bar; }
	cb.bounce += -jnbar*c.nMass;
	double vrnbar = -jnbar*c.nMass;
	cb.nMass += -jnbar*(c.bounce + vrn);
	double vrxbar = vrnbar*nx - vrtbar*ny;
	double vrybar = vrnbar*ny + vrtbar*nx;
	cb.nx += vrnbar*t.vrx + vrtbar*t.vry;
	cb.ny += vrnbar*t.vry - vrtbar*t.vrx;

	/* ---- bias impulse (bias velocities) ---- */
	double Bbx, Bby;
	adj_apply_pair(c, bx, by, A, B, true, Bbx, Bby, cb);
	double dbbar = Bbx*nx + Bby*ny;
	cb.nx += Bbx*db; cb.ny += Bby*db;
	double jB1bar = jBbar + dbbar, jB0bar = -dbbar;
	double jbnbar = 0.0;
	if(activeB){ jB0bar += jB1bar; jbnbar = jB1bar; }
	cb.bias += jbnbar*c.nMass;
	double vbnbar = -jbnbar*c.nMass;
	cb.nMass += jbnbar*(c.bias - vbn);
	cb.nx += vbnbar*t.vbx; cb.ny += vbnbar*t.vby;

	/* relative velocities -> body states before the application */
	adj_relvel(c, vrxbar, vrybar, t.wA, t.wB, A, B, false, cb);
	adj_relvel(c, vbnbar*nx, vbnbar*ny, t.wbA, t.wbB, A, B, true, cb);

	jNbar = jN0bar; jTbar = jT0bar; jBbar = jB0bar;
}

/* Reverse of the warm start of one contact (cpArbiter.c:441-455):
 * J = rotate(n, (jN, jT))*dt_coef applied as in app_adjoint. */
CPG_HD void warm_adjoint(const AdjCon &c, double jN, double jT, double dt_coef, const AdjBody &A, const AdjBody &B,
	double &jNbar, double &jTbar, AdjConBar &cb)
{
	double nx = c.nx, ny = c.ny;
	double jx = nx*jN - ny*jT, jy = nx*jT + ny*jN;
	double Jx = jx*dt_coef, Jy = jy*dt_coef;
	double Jbx, Jby;
	adj_apply_pair(c, Jx, Jy, A, B, false, Jbx, Jby, cb);
	double jxbar = Jbx*dt_coef, jybar = Jby*dt_coef;
	jNbar += jxbar*nx + jybar*ny;
	jTbar += -jxbar*ny + jybar*nx;
	cb.nx += jxbar*jN + jybar*jT;
	cb.ny += -jxbar*jT + jybar*jN;
}

/* Inputs of the pre-step of one contact (cpArbiter.c:416-439, with the
 * relative velocity of chipmunk_private.h:172-178 at the pre-step, i.e.
 * before the velocity integration). */
struct AdjPre {
	double r1x, r1y, r2x, r2y, nx, ny;
	double pAx, pAy, pBx, pBy;          /* body positions (after position integration) */
	double vAx, vAy, wA, vBx, vBy, wB;  /* velocities at the pre-step */
	double minvA, minvB, iinvA, iinvB;
	double e;                           /* arbiter elasticity */
	double biasCoef, slop, dt;
};

struct AdjPreBar {
	double r1x, r1y, r2x, r2y, nx, ny;
	double pAx, pAy, pBx, pBy;
	double vAx, vAy, wA, vBx, vBy, wB;
	double minvA, minvB, e;
};

CPG_HD void adj_zero(AdjPreBar &b)
{
	b.r1x = b.r1y = b.r2x = b.r2y = b.nx = b.ny = 0.0;
	b.pAx = b.pAy = b.pBx = b.pBy = 0.0;
	b.vAx = b.vAy = b.wA = b.vBx = b.vBy = b.wB = 0.0;
	b.minvA = b.minvB = b.e = 0.0;
}

/* Forward pre-step values (the device's k_build_rows expressions). */
CPG_HD void prestep_forward(const AdjPre &p, double &nMass, double &tMass, double &bias, double &bounce)
{
	double c1 = p.r1x*p.ny - p.r1y*p.nx, c2 = p.r2x*p.ny - p.r2y*p.nx;
	double kn = (p.minvA + p.iinvA*c1*c1) + (p.minvB + p.iinvB*c2*c2);
	nMass = 1.0/kn;
	double d1 = p.r1x*p.nx - p.r1y*(-p.ny), d2 = p.r2x*p.nx - p.r2y*(-p.ny);
	double kt = (p.minvA + p.iinvA*d1*d1) + (p.minvB + p.iinvB*d2*d2);
	tMass = 1.0/kt;
	double ddx = (p.r2x - p.r1x) + (p.pBx - p.pAx), ddy = (p.r2y - p.r1y) + (p.pBy - p.pAy);
	double dist = ddx*p.nx + ddy*p.ny;
	double x = dist + p.slop;
	double mn = (0.0 < x) ? 0.0 : x;
	bias = -p.biasCoef*mn/p.dt;
	double v1x = p.vAx + (-p.r1y)*p.wA, v1y = p.vAy + p.r1x*p.wA;
	double v2x = p.vBx + (-p.r2y)*p.wB, v2y = p.vBy + p.r2x*p.wB;
	double vrx = v2x - v1x, vry = v2y - v1y;
	bounce = (vrx*p.nx + vry*p.ny)*p.e;
}

/* Reverse of the pre-step: adjoints of nMass, tMass, bias, bounce -> the
 * inputs (accumulated into pb). */
CPG_HD void prestep_adjoint(const AdjPre &p, double nMassbar, double tMassbar, double biasbar, double bouncebar, AdjPreBar &pb)
{
	double nx = p.nx, ny = p.ny;
	/* nMass = 1/kn, kn = minvA + iinvA*c1^2 + minvB + iinvB*c2^2, c = r x n */
	double c1 = p.r1x*ny - p.r1y*nx, c2 = p.r2x*ny - p.r2y*nx;
	double kn = (p.minvA + p.iinvA*c1*c1) + (p.minvB + p.iinvB*c2*c2);
	double knbar = -nMassbar/(kn*kn);
	pb.minvA += knbar; pb.minvB += knbar;
	double c1bar = knbar*p.iinvA*2.0*c1, c2bar = knbar*p.iinvB*2.0*c2;
	pb.r1x += c1bar*ny; pb.r1y += -c1bar*nx; pb.nx += -c1bar*p.r1y; pb.ny += c1bar*p.r1x;
	pb.r2x += c2bar*ny; pb.r2y += -c2bar*nx; pb.nx += -c2bar*p.r2y; pb.ny += c2bar*p.r2x;
	/* tMass = 1/kt with the tangent: d = r x perp(n) = r . n */
	double d1 = p.r1x*nx - p.r1y*(-ny), d2 = p.r2x*nx - p.r2y*(-ny);
	double kt = (p.minvA + p.iinvA*d1*d1) + (p.minvB + p.iinvB*d2*d2);
	double ktbar = -tMassbar/(kt*kt);
	pb.minvA += ktbar; pb.minvB += ktbar;
	double d1bar = ktbar*p.iinvA*2.0*d1, d2bar = ktbar*p.iinvB*2.0*d2;
	pb.r1x += d1bar*nx; pb.r1y += d1bar*ny; pb.nx += d1bar*p.r1x; pb.ny += d1bar*p.r1y;
	pb.r2x += d2bar*nx; pb.r2y += d2bar*ny; pb.nx += d2bar*p.r2x; pb.ny += d2bar*p.r2y;
	/* bias = -biasCoef*min(0, dist + slop)/dt */
	double ddx = (p.r2x - p.r1x) + (p.pBx - p.pAx), ddy = (p.r2y - p.r1y) + (p.pBy - p.pAy);
	double dist = ddx*nx + ddy*ny;
	double distbar = (0.0 < dist + p.slop) ? 0.0 : biasbar*(-p.biasCoef)/p.dt;
	pb.r2x += distbar*nx; pb.r1x -= distbar*nx; pb.pBx += distbar*nx; pb.pAx -= distbar*nx;
	pb.r2y += distbar*ny; pb.r1y -= distbar*ny; pb.pBy += distbar*ny; pb.pAy -= distbar*ny;
	pb.nx += distbar*ddx; pb.ny += distbar*ddy;
	/* bounce = (vr . n)*e */
	double v1x = p.vAx + (-p.r1y)*p.wA, v1y = p.vAy + p.r1x*p.wA;
	double v2x = p.vBx + (-p.r2y)*p.wB, v2y = p.vBy + p.r2x*p.wB;
	double vrx = v2x - v1x, vry = v2y - v1y;
	double vrn = vrx*nx + vry*ny;
	pb.e += bouncebar*vrn;
	double vrnbar = bouncebar*p.e;
	double vrxbar = vrnbar*nx, vrybar = vrnbar*ny;
	pb.nx += vrnbar*vrx; pb.ny += vrnbar*vry;
	pb.vAx -= vrxbar; pb.vAy -= vrybar; pb.vBx += vrxbar; pb.vBy += vrybar;
	pb.wA += vrxbar*p.r1y - vrybar*p.r1x;
	pb.wB += -vrxbar*p.r2y + vrybar*p.r2x;
	pb.r1y += vrxbar*p.wA; pb.r1x += -vrybar*p.wA;
	pb.r2y += -vrxbar*p.wB; pb.r2x += vrybar*p.wB;
}

/* ---------------------------------------------------------------------
 * Contact geometry in dual numbers.  Component j of the derivative is
 * d/d(pose_j) for pose = (pA.x, pA.y, aA, pB.x, pB.y, aB).  A world point W
 * of a shape on a body at position p has dW/dp = I and dW/da = perp(W - p);
 * a world direction has dN/da = perp(N).  Values come from the forward's
 * world geometry, so the value parts below repeat the forward exactly.
 * ------------------------------------------------------------------- */
struct D6 { double v, d[6]; };
struct V2D { D6 x, y; };

CPG_HD D6 dconst(double v) { D6 r; r.v = v; for(int i = 0; i < 6; i++) r.d[i] = 0.0; return r; }
CPG_HD D6 dadd(const D6 &a, const D6 &b) { D6 r; r.v = a.v + b.v; for(int i = 0; i < 6; i++) r.d[i] = a.d[i] + b.d[i]; return r; }
CPG_HD D6 dsub(const D6 &a, const D6 &b) { D6 r; r.v = a.v - b.v; for(int i = 0; i < 6; i++) r.d[i] = a.d[i] - b.d[i]; return r; }
CPG_HD D6 dneg(const D6 &a) { D6 r; r.v = -a.v; for(int i = 0; i < 6; i++) r.d[i] = -a.d[i]; return r; }
CPG_HD D6 dmul(const D6 &a, const D6 &b) { D6 r; r.v = a.v*b.v; for(int i = 0; i < 6; i++) r.d[i] = a.d[i]*b.v + a.v*b.d[i]; return r; }
CPG_HD D6 dmuls(const D6 &a, double s) { D6 r; r.v = a.v*s; for(int i = 0; i < 6; i++) r.d[i] = a.d[i]*s; return r; }
CPG_HD D6 ddiv(const D6 &a, const D6 &b)
{
	D6 r; r.v = a.v/b.v;
	double ib = 1.0/b.v;
	for(int i = 0; i < 6; i++) r.d[i] = (a.d[i] - r.v*b.d[i])*ib;
	return r;
}
CPG_HD D6 dsqrt(const D6 &a)
{
	D6 r; r.v = sqrt(a.v);
	double h = (r.v > 0.0) ? 0.5/r.v : 0.0;
	for(int i = 0; i < 6; i++) r.d[i] = a.d[i]*h;
	return r;
}

CPG_HD V2D v2d(const D6 &x, const D6 &y) { V2D r; r.x = x; r.y = y; return r; }
CPG_HD V2D vdconst(double x, double y) { return v2d(dconst(x), dconst(y)); }
CPG_HD V2D vdadd(const V2D &a, const V2D &b) { return v2d(dadd(a.x, b.x), dadd(a.y, b.y)); }
CPG_HD V2D vdsub(const V2D &a, const V2D &b) { return v2d(dsub(a.x, b.x), dsub(a.y, b.y)); }
CPG_HD V2D vdneg(const V2D &a) { return v2d(dneg(a.x), dneg(a.y)); }
CPG_HD V2D vdmul(const V2D &a, const D6 &s) { return v2d(dmul(a.x, s), dmul(a.y, s)); }
CPG_HD V2D vdmuls(const V2D &a, double s) { return v2d(dmuls(a.x, s), dmuls(a.y, s)); }
CPG_HD D6 vddot(const V2D &a, const V2D &b) { return dadd(dmul(a.x, b.x), dmul(a.y, b.y)); }
CPG_HD D6 vdcross(const V2D &a, const V2D &b) { return dsub(dmul(a.x, b.y), dmul(a.y, b.x)); }
CPG_HD V2D vdrperp(const V2D &a) { return v2d(a.y, dneg(a.x)); }
CPG_HD D6 vdlensq(const V2D &a) { return vddot(a, a); }
CPG_HD V2D vdnormalize(const V2D &a) { return vdmul(a, ddiv(dconst(1.0), dadd(dsqrt(vdlensq(a)), dconst(DBL_MIN)))); }
/* cpvlerp(a, b, t) = a*(1 - t) + b*t */
CPG_HD V2D vdlerp(const V2D &a, const V2D &b, const D6 &t) { return vdadd(vdmul(a, dsub(dconst(1.0), t)), vdmul(b, t)); }
/* LerpT (cpCollision.c:203-206): a*(0.5 - t/2) + b*(0.5 + t/2) */
CPG_HD V2D vdlerp_t(const V2D &a, const V2D &b, const D6 &t)
{
	D6 ht = dmuls(t, 0.5);
	return vdadd(vdmul(a, dsub(dconst(0.5), ht)), vdmul(b, dadd(dconst(0.5), ht)));
}

/* A world point of a shape on body `side` (0: A, 1: B; -1: not moving). */
CPG_HD V2D world_point(double x, double y, double px, double py, int side)
{
	V2D r = vdconst(x, y);
	if(side >= 0){
		int o = 3*side;
		r.x.d[o] = 1.0; r.x.d[o + 2] = -(y - py);
		r.y.d[o + 1] = 1.0; r.y.d[o + 2] = x - px;
	}
	return r;
}

CPG_HD V2D world_dir(double x, double y, int side)
{
	V2D r = vdconst(x, y);
	if(side >= 0){ r.x.d[3*side + 2] = -y; r.y.d[3*side + 2] = x; }
	return r;
}

/* A shape's world geometry for the dual evaluation. */
struct GShape {
	int kind;                     /* 0 circle, 1 segment, 2 poly */
	int side;                     /* body slot in the dual (0/1), -1 if the body does not move */
	double px, py;                /* body position */
	double r;
	double p0x, p0y, p1x, p1y;    /* circle centre | segment ends (world) */
	double nx, ny;                /* segment normal (world) */
	int count;                    /* polygon vertex count */
	const double *vx, *vy, *wnx, *wny;   /* polygon world vertices and normals */
};

CPG_HD V2D gs_vertex(const GShape &s, int i)
{
	if(s.kind == 0) return world_point(s.p0x, s.p0y, s.px, s.py, s.side);
	if(s.kind == 1) return (i == 0) ? world_point(s.p0x, s.p0y, s.px, s.py, s.side) : world_point(s.p1x, s.p1y, s.px, s.py, s.side);
	int k = (i < s.count) ? i : 0;
	return world_point(s.vx[k], s.vy[k], s.px, s.py, s.side);
}

/* Up to two contacts: points on each shape and the shared normal. */
struct GContacts { int count; V2D n; V2D p1[2], p2[2]; };

CPG_HD void gc_push(GContacts &g, const V2D &p1, const V2D &p2)
{
	if(g.count < 2){ g.p1[g.count] = p1; g.p2[g.count] = p2; }
	g.count++;
}

CPG_HD double clamp01v(double f) { double m = (f < 1.0) ? f : 1.0; return (0.0 > m) ? 0.0 : m; }
CPG_HD D6 dclamp01(const D6 &f)
{
	/* value as dclamp01 (cpfclamp01); derivative zero when clamped */
	double v = clamp01v(f.v);
	if(v == f.v && f.v > 0.0 && f.v < 1.0) return f;
	if(v == f.v) return f;                 /* exactly at a bound, unclamped */
	return dconst(v);
}

/* ClosestT (cpCollision.c:199-201): -clamp(dot(b - a, a + b)/(|b - a|^2 + DBL_MIN), -1, 1) */
CPG_HD D6 dclosest_t(const V2D &a, const V2D &b)
{
	V2D delta = vdsub(b, a);
	D6 q = ddiv(vddot(delta, vdadd(a, b)), dadd(vdlensq(delta), dconst(DBL_MIN)));
	/* dclamp(q, -1, 1) = dmin(dmax(q, -1), 1) */
	double m = (q.v > -1.0) ? q.v : -1.0;
	D6 c = (q.v > -1.0) ? q : dconst(-1.0);
	if(!(m < 1.0)) c = dconst(1.0);
	return dneg(c);
}

struct GPts { V2D a, b, n; double d; double t; };

/* ClosestPointsNew (cpCollision.c:227-258) from the two Minkowski points
 * whose support indices the forward's final id encodes. */
CPG_HD GPts dclosest_points(const V2D &a0, const V2D &b0, const V2D &a1, const V2D &b1)
{
	V2D ab0 = vdsub(b0, a0), ab1 = vdsub(b1, a1);
	D6 t = dclosest_t(ab0, ab1);
	V2D p = vdlerp_t(ab0, ab1, t);
	GPts r;
	r.a = vdlerp_t(a0, a1, t);
	r.b = vdlerp_t(b0, b1, t);
	r.t = t.v;
	V2D delta = vdsub(ab1, ab0);
	V2D n = vdnormalize(vdrperp(delta));
	D6 d = vddot(n, p);
	if(d.v <= 0.0 || (-1.0 < t.v && t.v < 1.0)){
		r.n = n; r.d = d.v;
	} else {
		D6 d2 = dsqrt(vdlensq(p));
		r.n = vdmul(p, ddiv(dconst(1.0), dadd(d2, dconst(DBL_MIN))));
		r.d = d2.v;
	}
	return r;
}

struct GEdge { V2D a, b; double r; };

/* SupportEdgeForPoly (cpCollision.c:163-182); the choice uses values. */
CPG_HD GEdge dsupport_edge_poly(const GShape &s, const V2D &n)
{
	int count = s.count;
	double max = -INFINITY;
	int i1 = 0;
	for(int i = 0; i < count; i++){
		double d = s.vx[i]*n.x.v + s.vy[i]*n.y.v;
		if(d > max){ max = d; i1 = i; }
	}
	int i0 = (i1 - 1 + count)%count, i2 = (i1 + 1)%count;
	GEdge e;
	e.r = s.r;
	double d1 = n.x.v*s.wnx[i1] + n.y.v*s.wny[i1], d2 = n.x.v*s.wnx[i2] + n.y.v*s.wny[i2];
	if(d1 > d2){ e.a = gs_vertex(s, i0); e.b = gs_vertex(s, i1); }
	else { e.a = gs_vertex(s, i1); e.b = gs_vertex(s, i2); }
	return e;
}

/* SupportEdgeForSegment (cpCollision.c:184-195). */
CPG_HD GEdge dsupport_edge_segment(const GShape &s, const V2D &n)
{
	GEdge e;
	e.r = s.r;
	if(s.nx*n.x.v + s.ny*n.y.v > 0.0){ e.a = gs_vertex(s, 0); e.b = gs_vertex(s, 1); }
	else { e.a = gs_vertex(s, 1); e.b = gs_vertex(s, 0); }
	return e;
}

/* ContactPoints (cpCollision.c:477-518). */
CPG_HD void dcontact_points(const GEdge &e1, const GEdge &e2, const GPts &pts, GContacts &g)
{
	double mindist = e1.r + e2.r;
	if(pts.d <= mindist){
		V2D n = g.n = pts.n;
		D6 d_e1_a = vdcross(e1.a, n), d_e1_b = vdcross(e1.b, n);
		D6 d_e2_a = vdcross(e2.a, n), d_e2_b = vdcross(e2.b, n);
		D6 e1_denom = ddiv(dconst(1.0), dadd(dsub(d_e1_b, d_e1_a), dconst(DBL_MIN)));
		D6 e2_denom = ddiv(dconst(1.0), dadd(dsub(d_e2_b, d_e2_a), dconst(DBL_MIN)));
		{
			V2D p1 = vdadd(vdmuls(n, e1.r), vdlerp(e1.a, e1.b, dclamp01(dmul(dsub(d_e2_b, d_e1_a), e1_denom))));
			V2D p2 = vdadd(vdmuls(n, -e2.r), vdlerp(e2.a, e2.b, dclamp01(dmul(dsub(d_e1_a, d_e2_a), e2_denom))));
			D6 dist = vddot(vdsub(p2, p1), n);
			if(dist.v <= 0.0) gc_push(g, p1, p2);
		}{
			V2D p1 = vdadd(vdmuls(n, e1.r), vdlerp(e1.a, e1.b, dclamp01(dmul(dsub(d_e2_a, d_e1_a), e1_denom))));
			V2D p2 = vdadd(vdmuls(n, -e2.r), vdlerp(e2.a, e2.b, dclamp01(dmul(dsub(d_e1_b, d_e2_a), e2_denom))));
			D6 dist = vddot(vdsub(p2, p1), n);
			if(dist.v <= 0.0) gc_push(g, p1, p2);
		}
	}
}

/* The contacts of a pair (shapes ordered by kind, as the forward's arbiter
 * stores them), with derivatives.  `id` is the forward's final GJK id. */
CPG_HD void geom_contacts(const GShape &A, const GShape &B, unsigned id, GContacts &g)
{
	g.count = 0;
	g.n = vdconst(0.0, 0.0);
	int pair = A.kind + B.kind*3;
	if(pair == 0){
		/* CircleToCircle, cpCollision.c:525-537 */
		V2D c1 = gs_vertex(A, 0), c2 = gs_vertex(B, 0);
		double mindist = A.r + B.r;
		V2D delta = vdsub(c2, c1);
		D6 distsq = vdlensq(delta);
		if(distsq.v < mindist*mindist){
			D6 dist = dsqrt(distsq);
			V2D n = dist.v ? vdmul(delta, ddiv(dconst(1.0), dist)) : vdconst(1.0, 0.0);
			g.n = n;
			gc_push(g, vdadd(c1, vdmuls(n, A.r)), vdadd(c2, vdmuls(n, -B.r)));
		}
		return;
	}
	if(pair == 3){
		/* CircleToSegment, cpCollision.c:539-569 (the forward pushed the
		 * contact, so the end-cap test passed) */
		V2D seg_a = gs_vertex(B, 0), seg_b = gs_vertex(B, 1), center = gs_vertex(A, 0);
		V2D seg_delta = vdsub(seg_b, seg_a);
		D6 ct = dclamp01(ddiv(vddot(seg_delta, vdsub(center, seg_a)), vdlensq(seg_delta)));
		V2D closest = vdadd(seg_a, vdmul(seg_delta, ct));
		double mindist = A.r + B.r;
		V2D delta = vdsub(closest, center);
		D6 distsq = vdlensq(delta);
		if(distsq.v < mindist*mindist){
			D6 dist = dsqrt(distsq);
			V2D n = dist.v ? vdmul(delta, ddiv(dconst(1.0), dist)) : world_dir(B.nx, B.ny, B.side);
			g.n = n;
			gc_push(g, vdadd(center, vdmuls(n, A.r)), vdadd(closest, vdmuls(n, -B.r)));
		}
		return;
	}
	/* GJK-based pairs: the final Minkowski edge from the id */
	V2D a0 = gs_vertex(A, (id >> 24) & 0xFF), b0 = gs_vertex(B, (id >> 16) & 0xFF);
	V2D a1 = gs_vertex(A, (id >> 8) & 0xFF), b1 = gs_vertex(B, id & 0xFF);
	GPts pts = dclosest_points(a0, b0, a1, b1);
	if(pair == 6){
		/* CircleToPoly, cpCollision.c:661-679 */
		if(pts.d <= A.r + B.r){
			g.n = pts.n;
			gc_push(g, vdadd(pts.a, vdmuls(pts.n, A.r)), vdadd(pts.b, vdmuls(pts.n, -B.r)));
		}
	} else if(pair == 4){
		/* SegmentToSegment, cpCollision.c:571-604 */
		if(pts.d <= A.r + B.r) dcontact_points(dsupport_edge_segment(A, pts.n), dsupport_edge_segment(B, vdneg(pts.n)), pts, g);
	} else if(pair == 7){
		/* SegmentToPoly, cpCollision.c:629-659 */
		if(pts.d - A.r - B.r <= 0.0) dcontact_points(dsupport_edge_segment(A, pts.n), dsupport_edge_poly(B, vdneg(pts.n)), pts, g);
	} else if(pair == 8){
		/* PolyToPoly, cpCollision.c:606-627 */
		if(pts.d - A.r - B.r <= 0.0) dcontact_points(dsupport_edge_poly(A, pts.n), dsupport_edge_poly(B, vdneg(pts.n)), pts, g);
	}
}

/* Reverse through the contact geometry: with r1 = p1 - pA, r2 = p2 - pB
 * and n, the adjoints r1bar[k], r2bar[k] (per contact) and nbar give the
 * pose adjoints poseBar[6] (added). */
CPG_HD void geom_adjoint(const GContacts &g, int count, const double *r1bar, const double *r2bar, double nbx, double nby, double *poseBar)
{
	for(int j = 0; j < 6; j++) poseBar[j] += nbx*g.n.x.d[j] + nby*g.n.y.d[j];
	for(int k = 0; k < count && k < 2; k++){
		for(int j = 0; j < 6; j++){
			poseBar[j] += r1bar[2*k]*g.p1[k].x.d[j] + r1bar[2*k + 1]*g.p1[k].y.d[j];
			poseBar[j] += r2bar[2*k]*g.p2[k].x.d[j] + r2bar[2*k + 1]*g.p2[k].y.d[j];
		}
		poseBar[0] -= r1bar[2*k]; poseBar[1] -= r1bar[2*k + 1];
		poseBar[3] -= r2bar[2*k]; poseBar[4] -= r2bar[2*k + 1];
	}
}

/* ---------------------------------------------------------------------
 * Four lanes per contact for the reverse of an application, as the
 * forward solve runs it: lane q takes side q & 1 (0: body a, 1: body b)
 * and part q >> 1 (0: velocity with the normal and friction impulse,
 * 1: bias velocity with the bias impulse).  The two parts touch disjoint
 * state.  Within a part, each lane computes its body's share of the
 * impulse adjoint (phase 1); the shares are added across the pair (a
 * shuffle on the device); both lanes then run the scalar part and update
 * their own body (phase 2).
 *
 * Every lane runs the same instructions: the part and side pick operands
 * (selects and sign flips of the bit pattern), never branches, because a
 * warp that diverges on them issues both paths and each double-precision
 * instruction is issued once per warp whatever its active lanes.  The bias
 * part is the velocity part with no friction (its friction impulse is the
 * constant 0).  Clamp activity is read from the recorded results: a
 * normal or bias accumulator clamps at 0 exactly when its result is +0,
 * and the friction clamp took the bound whose bit pattern the result
 * carries (dclamp returns one of its operands), which is the forward's
 * branch exactly.
 *
 * The constants' adjoints go to per-lane partial sums (AdjLaneBar): each
 * lane sums 1/m and r of its own body; the contact's scalars, which both
 * lanes of a part could compute, are split between them (side 0: n.x,
 * tMass and the constant term; side 1: n.y, u and nMass), so each lane
 * issues half of those operations.  lane_bar_sum turns the four lanes'
 * sums into the contact's AdjConBar, equal to app_adjoint's up to the
 * order of the additions.
 * ------------------------------------------------------------------- */
CPG_HD long long adj_bits(double x)
{
#ifdef __CUDA_ARCH__
	return __double_as_longlong(x);
#else
	long long b; memcpy(&b, &x, sizeof(b)); return b;
#endif
}

CPG_HD double adj_double(long long b)
{
#ifdef __CUDA_ARCH__
	return __longlong_as_double(b);
#else
	double x; memcpy(&x, &b, sizeof(x)); return x;
#endif
}

#define ADJ_SIGN ((long long)0x8000000000000000ULL)

CPG_HD double adj_neg_if(double x, bool f) { return adj_double(adj_bits(x) ^ (f ? ADJ_SIGN : 0LL)); }

/* The lane's constants: its body's 1/m, 1/I, r; the part's constant term
 * (bounce for the velocity part, bias for the bias part). */
struct AdjLane {
	int side, part;
	double nx, ny, minv, iinv, rx, ry, c0, nMass, tMass, u;
};

/* The lane's view of a record: the part's accumulator before and after
 * (J0, J1), friction before and after (T0, T1: 0 for the bias part), the
 * part's relative velocity and the lane's body's angular velocity. */
struct AdjLaneRec { double J0, J1, T0, T1, vrx, vry, wown; };

/* Per-lane partial sums of the contact's constants' adjoints (1/m and r of
 * the lane's body; the scalars split by side: n.x, tMass, c0 on side 0,
 * n.y, u, nMass on side 1), and the accumulator adjoints the part carries
 * (velocity: jA = jN, j2 = jT; bias: jA = jB). */
struct alignas(16) AdjLaneBar { double minv, rx, ry, nx, ny, tMass, u, c0, nMass, jA, j2, pad; };

CPG_HD void lane_bar_zero(AdjLaneBar &b)
{
	b.minv = b.rx = b.ry = b.nx = b.ny = b.tMass = b.u = b.c0 = b.nMass = b.jA = b.j2 = b.pad = 0.0;
}

CPG_HD AdjLane adj_lane(const AdjCon &c, int q)
{
	AdjLane L;
	L.side = q & 1; L.part = q >> 1;
	L.nx = c.nx; L.ny = c.ny;
	L.minv = L.side ? c.minvB : c.minvA;
	L.iinv = L.side ? c.iinvB : c.iinvA;
	L.rx = L.side ? c.r2x : c.r1x;
	L.ry = L.side ? c.r2y : c.r1y;
	L.c0 = L.part ? c.bias : c.bounce;
	L.nMass = c.nMass; L.tMass = c.tMass; L.u = c.u;
	return L;
}

CPG_HD AdjLaneRec adj_lane_rec(const AdjApp &t, int side, int part)
{
	const double *p = &t.jN0;     /* AdjApp is 14 consecutive doubles */
	AdjLaneRec r;
	r.J0 = p[part ? 2 : 0]; r.J1 = p[part ? 5 : 3];
	r.T0 = part ? 0.0 : p[1]; r.T1 = part ? 0.0 : p[4];
	r.vrx = p[part ? 8 : 6]; r.vry = p[part ? 9 : 7];
	r.wown = p[10 + 2*part + side];
	return r;
}

/* Phase 1: the lane's share (jbx, jby) of the adjoint of the part's
 * impulse, from its body's adjoint (ax, ay, aw) after the application. */
CPG_HD void lane_adj_phase1(const AdjLane &L, const AdjLaneRec &t, double ax, double ay, double aw,
	double &jbx, double &jby, AdjLaneBar &b)
{
	double dN = t.J1 - t.J0, dT = t.T1 - t.T0;
	double Jx = L.nx*dN - L.ny*dT, Jy = L.nx*dT + L.ny*dN;
	bool neg = (L.side == 0);                /* b receives J, a receives -J */
	double sminv = adj_neg_if(L.minv, neg), siinv = adj_neg_if(L.iinv, neg);
	jbx = sminv*ax; jby = sminv*ay;
	double gm = adj_neg_if(Jx*ax + Jy*ay, neg);
	double g = siinv*aw;
	b.minv += gm; b.rx += g*Jy; b.ry -= g*Jx;
	jbx += -g*L.ry; jby += g*L.rx;
}

/* Phase 2, scalar part: with the pair's total (Jbx, Jby), the adjoints of
 * the part's accumulators (b.jA, b.j2, after to before) and of the
 * contact's scalars, and the adjoint (dbx, dby) of the part's relative
 * velocity.  The scalars' partial sums are split by side: a side-0 lane
 * sums n.x, tMass and the constant term (bounce or bias), a side-1 lane
 * n.y, u and nMass.  With BOTH (one lane for both sides) the side-1 sums
 * go to *b1. */
template<bool BOTH>
CPG_HD void lane_adj_scalar_t(const AdjLane &L, const AdjLaneRec &t, double Jbx, double Jby,
	double &dbx, double &dby, AdjLaneBar &b, AdjLaneBar *b1)
{
	double nx = L.nx, ny = L.ny;
	bool vel = (L.part == 0);
	bool s1 = !BOTH && L.side == 1;
	double dN = t.J1 - t.J0, dT = t.T1 - t.T0;
	double vn = t.vrx*nx + t.vry*ny;
	double vt = t.vry*nx - t.vrx*ny;
	double dNbar = Jbx*nx + Jby*ny;
	double dTbar = Jby*nx - Jbx*ny;
	double J1bar = b.jA + dNbar, J0bar = -dNbar;
	double T1bar = b.j2 + dTbar, T0bar = -dTbar;
	/* friction: dclamp(f, -jtMax, jtMax) returned f, -jtMax or jtMax */
	double jtMax = L.u*t.J1;
	long long bt = adj_bits(t.T1), bm = adj_bits(jtMax);
	bool top = (bt == bm), bot = !top && (bt == (bm ^ ADJ_SIGN));
	double fbar = (vel && !top && !bot) ? T1bar : 0.0;
	double mbar = (vel && (top || bot)) ? adj_neg_if(T1bar, bot) : 0.0;
	T0bar += fbar;
	double vtbar = -fbar*L.tMass;
	J1bar += mbar*L.u;
	/* normal (bias): dmax(J0 + j, 0) passed J0 + j on when the result is not +0 */
	double jnbar = (adj_bits(t.J1) > 0) ? J1bar : 0.0;
	J0bar += jnbar;
	/* j = y*nMass with y = -(bounce + vn) (velocity) or bias - vn (bias) */
	double y = adj_neg_if(L.c0 + adj_neg_if(vn, !vel), vel);
	double vnbar = -jnbar*L.nMass;
	dbx = vnbar*nx - vtbar*ny; dby = vnbar*ny + vtbar*nx;
	/* n.x: Jb.(dN, dT) rotated + vnbar vr + vtbar perp; n.y likewise */
	if(BOTH){
		b.nx += Jbx*dN + Jby*dT;
		b.nx += vnbar*t.vrx + vtbar*t.vry;
		b.tMass -= fbar*vt;
		b.c0 += adj_neg_if(jnbar, vel)*L.nMass;
		b1->ny += Jby*dN - Jbx*dT;
		b1->ny += vnbar*t.vry - vtbar*t.vrx;
		b1->u += mbar*t.J1;
		b1->nMass += jnbar*y;
	} else {
		double n = s1 ? b.ny : b.nx;
		n += (s1 ? Jby : Jbx)*dN + (s1 ? -Jbx : Jby)*dT;
		n += vnbar*(s1 ? t.vry : t.vrx) + vtbar*(s1 ? -t.vrx : t.vry);
		double tu = s1 ? b.u : b.tMass;
		tu += (s1 ? mbar : -fbar)*(s1 ? t.J1 : vt);
		double cn = s1 ? b.nMass : b.c0;
		cn += (s1 ? jnbar : adj_neg_if(jnbar, vel))*(s1 ? y : L.nMass);
		if(s1){ b.ny = n; b.u = tu; b.nMass = cn; }
		else { b.nx = n; b.tMass = tu; b.c0 = cn; }
	}
	b.jA = J0bar; b.j2 = T0bar;
}

CPG_HD void lane_adj_scalar(const AdjLane &L, const AdjLaneRec &t, double Jbx, double Jby,
	double &dbx, double &dby, AdjLaneBar &b)
{
	lane_adj_scalar_t<false>(L, t, Jbx, Jby, dbx, dby, b, nullptr);
}

/* Phase 2, body part: the adjoint of one body's velocity through the
 * relative velocity d = (v_b + perp(r2) w_b) - (v_a + perp(r1) w_a), and
 * of its r. */
CPG_HD void lane_adj_body(int side, double rx, double ry, double wown, double dbx, double dby,
	double &ax, double &ay, double &aw, AdjLaneBar &b)
{
	bool neg = (side == 0);
	double sdx = adj_neg_if(dbx, neg), sdy = adj_neg_if(dby, neg);
	ax += sdx; ay += sdy;
	aw += rx*sdy - ry*sdx;
	b.ry -= sdx*wown; b.rx += sdy*wown;
}

/* Phase 2 on a four-lane quad: the scalar part (both lanes of a part
 * compute it; side 0's sums are the ones used), then the lane's own body. */
CPG_HD void lane_adj_phase2(const AdjLane &L, const AdjLaneRec &t, double Jbx, double Jby,
	double &ax, double &ay, double &aw, AdjLaneBar &b)
{
	double dbx, dby;
	lane_adj_scalar(L, t, Jbx, Jby, dbx, dby, b);
	lane_adj_body(L.side, L.rx, L.ry, t.wown, dbx, dby, ax, ay, aw, b);
}

/* Two lanes per contact: lane p takes part p for both bodies (La, Lb:
 * the part's side-0 and side-1 lanes' constants, wa, wb: the bodies'
 * recorded angular velocities of the part).  Ba collects the contact's
 * scalars and the part's accumulator adjoints like a side-0 lane, Bb the
 * side-1 body's 1/m and r; the other fields of Bb are not used. */
CPG_HD void pair_adj_apply(const AdjLane &La, const AdjLane &Lb, const AdjLaneRec &t, double wa, double wb,
	double &ax, double &ay, double &aw, double &bx, double &by, double &bw, AdjLaneBar &Ba, AdjLaneBar &Bb)
{
	double dN = t.J1 - t.J0, dT = t.T1 - t.T0;
	double Jx = La.nx*dN - La.ny*dT, Jy = La.nx*dT + La.ny*dN;
	double gmJ_a = Jx*ax + Jy*ay, gmJ_b = Jx*bx + Jy*by;
	/* side a receives -J, side b receives J */
	double ga = -(La.iinv*aw), gb = Lb.iinv*bw;
	double jbx = (-La.minv)*ax + Lb.minv*bx;
	double jby = (-La.minv)*ay + Lb.minv*by;
	Ba.minv -= gmJ_a; Bb.minv += gmJ_b;
	Ba.rx += ga*Jy; Ba.ry -= ga*Jx;
	Bb.rx += gb*Jy; Bb.ry -= gb*Jx;
	jbx += -ga*La.ry - gb*Lb.ry;
	jby += ga*La.rx + gb*Lb.rx;
	double dbx, dby;
	lane_adj_scalar_t<true>(La, t, jbx, jby, dbx, dby, Ba, &Bb);
	lane_adj_body(0, La.rx, La.ry, wa, dbx, dby, ax, ay, aw, Ba);
	lane_adj_body(1, Lb.rx, Lb.ry, wb, dbx, dby, bx, by, bw, Bb);
}

/* Warm start on the two velocity lanes: phase 1 as for an application
 * with J = rotate(n, (jN, jT))*dt_coef. */
CPG_HD void lane_warm_phase1(const AdjLane &L, double jN, double jT, double dt_coef, double ax, double ay, double aw,
	double &jbx, double &jby, AdjLaneBar &b)
{
	double jx = L.nx*jN - L.ny*jT, jy = L.nx*jT + L.ny*jN;
	double Jx = jx*dt_coef, Jy = jy*dt_coef;
	bool neg = (L.side == 0);
	double sminv = adj_neg_if(L.minv, neg), siinv = adj_neg_if(L.iinv, neg);
	jbx = sminv*ax; jby = sminv*ay;
	double gm = adj_neg_if(Jx*ax + Jy*ay, neg);
	double g = siinv*aw;
	b.minv += gm; b.rx += g*Jy; b.ry -= g*Jx;
	jbx += -g*L.ry; jby += g*L.rx;
}

CPG_HD void lane_warm_phase2(const AdjLane &L, double jN, double jT, double dt_coef, double Jbx, double Jby, AdjLaneBar &b)
{
	double jxbar = Jbx*dt_coef, jybar = Jby*dt_coef;
	b.jA += jxbar*L.nx + jybar*L.ny;
	b.j2 += jybar*L.nx - jxbar*L.ny;
	/* side 0 sums n.x, side 1 n.y */
	bool s1 = L.side == 1;
	double n = s1 ? b.ny : b.nx;
	n += (s1 ? jybar : jxbar)*jN + (s1 ? -jxbar : jybar)*jT;
	if(s1) b.ny = n; else b.nx = n;
}

/* The contact's constants' adjoints from its four lanes' partial sums
 * (lanes 0, 1: velocity part, sides a, b; lanes 2, 3: bias part). */
CPG_HD void lane_bar_sum(const AdjLaneBar *l, AdjConBar &cb)
{
	cb.minvA = l[0].minv + l[2].minv; cb.minvB = l[1].minv + l[3].minv;
	cb.r1x = l[0].rx + l[2].rx; cb.r1y = l[0].ry + l[2].ry;
	cb.r2x = l[1].rx + l[3].rx; cb.r2y = l[1].ry + l[3].ry;
	cb.nx = l[0].nx + l[2].nx; cb.ny = l[1].ny + l[3].ny;
	cb.nMass = l[1].nMass + l[3].nMass;
	cb.tMass = l[0].tMass; cb.u = l[1].u;
	cb.bounce = l[0].c0; cb.bias = l[2].c0;
}
