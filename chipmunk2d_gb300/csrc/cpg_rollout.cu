/*
 * cpg_rollout.cu -- recording and reverse pass of the differentiable
 * rollout (reference-order mode, batched worlds).
 *
 * The forward rollout keeps a copy of the whole device set every K steps.
 * The reverse pass restores each checkpoint, replays its K steps with
 * recording on (k_tape_*: positions after integration, pre-step
 * velocities, world geometry, the pre-step rows with their arbiter data,
 * the level structure, and per impulse application the accumulators and
 * velocities the solver saw, written by the solve kernel itself), then
 * runs k_adj_step for the K steps in reverse.
 *
 * k_adj_step, one block per world, reverses one step (cpSpaceStep.c:
 * 335-445) in the opposite order of the forward:
 *   1. the adjoints of the impulses stored in the arbiters at the end of
 *      the step seed the contacts' accumulators;
 *   2. the iterations in reverse, levels in reverse (units of one level
 *      touch disjoint dynamic bodies, so they run in parallel without
 *      conflicts), contacts of a unit in reverse (app_adjoint);
 *   3. the warm start (warm_adjoint); the adjoints of the initial
 *      accumulators go to the arbiter contacts they were copied from
 *      (cpArbiterUpdate's hash match);
 *   4. velocity integration (damping) and the bias velocities, which the
 *      step starts at zero;
 *   5. pre-step (prestep_adjoint) and contact geometry (geom_contacts in
 *      dual numbers, geom_adjoint) per unit, by levels;
 *   6. position integration, which turns the pose adjoints into those of
 *      the previous step's velocities and bias velocities.
 * Parameter gradients: 1/m per body (impulses, pre-step masses), and the
 * arbiter's e and u, split onto the two shapes (e = ea*eb, u = ua*ub).
 * External forces are not differentiated (the rollout scenes have none).
 */
#include <cuda_runtime.h>
#include "cpg_device.h"
#include "cpg_adjoint.cuh"

enum { ROW_FIRST_ = 1, ROW_DYN_A_ = 2, ROW_DYN_B_ = 4 };

/* ---- recording ---- */

/* Per-world offsets of this step's rows and level starts in the tape. */
__global__ void k_tape_offsets(cpgSet s)
{
	__shared__ int warpSums[2][32];
	__shared__ int carry[2];
	cpgTape &tp = s.tape;
	int t = tp.step, nw = s.nworlds;
	int *rowOff = tp.rowOff + (size_t)t*(nw + 1);
	int *levOff = tp.levOff + (size_t)t*(nw + 1);
	if(threadIdx.x == 0){ carry[0] = tp.cursor[0]; carry[1] = tp.cursor[1]; }
	__syncthreads();
	int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
	for(int c0 = 0; c0 < nw; c0 += blockDim.x){
		int w = c0 + threadIdx.x;
		int nr = 0, nl = 0;
		if(w < nw){
			bool active = s.params[w].active != 0;
			const cpgTree &T = s.tree[w];
			nr = active ? T.nunits : 0;
			nl = active ? T.nlevels + 1 : 0;
			tp.params[(size_t)t*nw + w] = s.params[w];
		}
		int xr = nr, xl = nl;
		for(int o = 1; o < 32; o <<= 1){
			int yr = __shfl_up_sync(0xffffffffu, xr, o), yl = __shfl_up_sync(0xffffffffu, xl, o);
			if(lane >= o){ xr += yr; xl += yl; }
		}
		if(lane == 31){ warpSums[0][warp] = xr; warpSums[1][warp] = xl; }
		__syncthreads();
		if(warp == 0){
			int a = (lane < nwarps) ? warpSums[0][lane] : 0, b = (lane < nwarps) ? warpSums[1][lane] : 0;
			for(int o = 1; o < 32; o <<= 1){
				int ya = __shfl_up_sync(0xffffffffu, a, o), yb = __shfl_up_sync(0xffffffffu, b, o);
				if(lane >= o){ a += ya; b += yb; }
			}
			if(lane < nwarps){ warpSums[0][lane] = a; warpSums[1][lane] = b; }
		}
		__syncthreads();
		int pr = (warp > 0) ? warpSums[0][warp - 1] : 0, pl = (warp > 0) ? warpSums[1][warp - 1] : 0;
		if(w < nw){ rowOff[w] = carry[0] + pr + xr - nr; levOff[w] = carry[1] + pl + xl - nl; }
		__syncthreads();
		if(threadIdx.x == 0){ carry[0] += warpSums[0][nwarps - 1]; carry[1] += warpSums[1][nwarps - 1]; }
		__syncthreads();
	}
	if(threadIdx.x == 0){
		rowOff[nw] = carry[0]; levOff[nw] = carry[1];
		tp.cursor[0] = carry[0]; tp.cursor[1] = carry[1];
		if(carry[0] > tp.rowCap || carry[1] > tp.levCap) tp.cursor[2] = 1;
	}
}

__global__ void k_tape_bodies(cpgSet s)
{
	int g = blockIdx.x*blockDim.x + threadIdx.x;
	int nb = s.totalBodies;
	if(g >= nb) return;
	double *b = s.tape.body + (size_t)s.tape.step*8*nb;
	b[g] = s.px[g]; b[nb + g] = s.py[g]; b[2*(size_t)nb + g] = s.ang[g];
	b[3*(size_t)nb + g] = s.vx[g]; b[4*(size_t)nb + g] = s.vy[g]; b[5*(size_t)nb + g] = s.w[g];
	b[6*(size_t)nb + g] = s.ta[g]; b[7*(size_t)nb + g] = s.tb[g];
}

__global__ void k_tape_shapes(cpgSet s)
{
	int g = blockIdx.x*blockDim.x + threadIdx.x;
	int ns = s.totalShapes, nv = s.totalVerts;
	if(g < ns){
		double *p = s.tape.shape + (size_t)s.tape.step*6*ns;
		p[g] = s.w0x[g]; p[ns + g] = s.w0y[g]; p[2*(size_t)ns + g] = s.w1x[g];
		p[3*(size_t)ns + g] = s.w1y[g]; p[4*(size_t)ns + g] = s.wnx[g]; p[5*(size_t)ns + g] = s.wny[g];
	}
	if(g < nv){
		double *v = s.tape.verts + (size_t)s.tape.step*4*nv;
		v[g] = s.gvx[g]; v[nv + g] = s.gvy[g]; v[2*(size_t)nv + g] = s.gnx[g]; v[3*(size_t)nv + g] = s.gny[g];
	}
}

__global__ void k_tape_rows(cpgSet s)
{
	int w = blockIdx.y;
	const cpgTape &tp = s.tape;
	int nw = s.nworlds, t = tp.step;
	if(!s.params[w].active) return;
	const cpgWorld &W = s.world[w];
	const cpgTree &T = s.tree[w];
	int ro = tp.rowOff[(size_t)t*(nw + 1) + w], lo = tp.levOff[(size_t)t*(nw + 1) + w];
	int n = T.nunits, nl = T.nlevels + 1;
	const int *start = s.levelStart + W.unitOff + w;
	for(int k = blockIdx.x*blockDim.x + threadIdx.x; k < n; k += gridDim.x*blockDim.x){
		if(ro + k >= tp.rowCap) break;
		const cpgRow &row = s.rows[W.unitOff + k];
		tp.rows[ro + k] = row;
		int *info = tp.rowInfo + 4*(size_t)(ro + k);
		if(row.kind == 0){
			const cpgArb &arb = s.arbs[row.src];
			info[0] = arb.a; info[1] = arb.b; info[2] = (int)arb.gjk; info[3] = arb.warmSrc;
		} else {
			info[0] = -1; info[1] = -1; info[2] = 0; info[3] = 0;
		}
	}
	for(int l = blockIdx.x*blockDim.x + threadIdx.x; l < nl; l += gridDim.x*blockDim.x)
		if(lo + l < tp.levCap) tp.levels[lo + l] = start[l];
}

static inline int blocks_of(int n, int bs) { return (n + bs - 1)/bs > 0 ? (n + bs - 1)/bs : 1; }

extern "C" int cpg_launch_tape(const cpgSet *s, void *stream)
{
	cudaStream_t st = (cudaStream_t)stream;
	k_tape_offsets<<<1, 1024, 0, st>>>(*s);
	k_tape_bodies<<<blocks_of(s->totalBodies, 256), 256, 0, st>>>(*s);
	int nsv = s->totalShapes > s->totalVerts ? s->totalShapes : s->totalVerts;
	k_tape_shapes<<<blocks_of(nsv, 256), 256, 0, st>>>(*s);
	k_tape_rows<<<dim3(1, s->nworlds), 128, 0, st>>>(*s);
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}

/* ---- reverse pass ---- */

struct AdjScratch { AdjConBar cb; double jN, jT, jB; };

__device__ __forceinline__ AdjScratch *con_scratch(const cpgAdj &a, size_t row, int c)
{
	return (AdjScratch *)(a.con + (row*2 + (size_t)c)*16);
}

__device__ __forceinline__ AdjBody load_bar(const cpgAdj &a, int g)
{
	const double *b = a.body + 9*(size_t)g;
	AdjBody r; r.vx = b[3]; r.vy = b[4]; r.w = b[5]; r.vbx = b[6]; r.vby = b[7]; r.wb = b[8];
	return r;
}

__device__ __forceinline__ void store_bar(const cpgAdj &a, int g, const AdjBody &r)
{
	double *b = a.body + 9*(size_t)g;
	b[3] = r.vx; b[4] = r.vy; b[5] = r.w; b[6] = r.vbx; b[7] = r.vby; b[8] = r.wb;
}

__device__ __forceinline__ AdjCon make_con(const cpgSet &s, const cpgRow &row, int c, int ga, int gb)
{
	const cpgRowContact &rc = row.arb.c[c];
	AdjCon k;
	k.r1x = rc.r1x; k.r1y = rc.r1y; k.r2x = rc.r2x; k.r2y = rc.r2y;
	k.nx = row.arb.nx; k.ny = row.arb.ny;
	k.nMass = rc.nMass; k.tMass = rc.tMass; k.bias = rc.bias; k.bounce = rc.bounce; k.u = row.arb.u;
	k.minvA = s.minv[ga]; k.minvB = s.minv[gb]; k.iinvA = s.iinv[ga]; k.iinvB = s.iinv[gb];
	return k;
}

/* A shape's recorded world geometry at step t as a GShape. */
__device__ GShape tape_gshape(const cpgSet &s, int t, int g, int bodyG, int side)
{
	const cpgTape &tp = s.tape;
	int ns = s.totalShapes, nv = s.totalVerts, nb = s.totalBodies;
	const double *sh = tp.shape + (size_t)t*6*ns;
	const double *bd = tp.body + (size_t)t*8*nb;
	GShape r;
	r.kind = s.skind[g];
	r.side = side;
	r.px = bd[bodyG]; r.py = bd[nb + bodyG];
	r.r = s.sr[g];
	r.p0x = sh[g]; r.p0y = sh[ns + g]; r.p1x = sh[2*(size_t)ns + g]; r.p1y = sh[3*(size_t)ns + g];
	r.nx = sh[4*(size_t)ns + g]; r.ny = sh[5*(size_t)ns + g];
	r.count = s.svcount[g];
	int voff = s.world[s.sworld[g]].vertOff + s.svoff[g];
	const double *vt = tp.verts + (size_t)t*4*nv;
	r.vx = vt + voff; r.vy = vt + nv + voff; r.wnx = vt + 2*(size_t)nv + voff; r.wny = vt + 3*(size_t)nv + voff;
	return r;
}

__global__ void k_adj_step(cpgSet s, cpgAdj a, int t)
{
	int w = blockIdx.x;
	const cpgTape &tp = s.tape;
	int nw = s.nworlds;
	const cpgParams P = tp.params[(size_t)t*nw + w];
	if(!P.active) return;
	const cpgWorld &W = s.world[w];
	int ro = tp.rowOff[(size_t)t*(nw + 1) + w];
	int n = tp.rowOff[(size_t)t*(nw + 1) + w + 1] - ro;
	int lo = tp.levOff[(size_t)t*(nw + 1) + w];
	int nlev = tp.levOff[(size_t)t*(nw + 1) + w + 1] - lo - 1;
	const int *start = tp.levels + lo;
	const cpgRow *rows = tp.rows + ro;
	const int *info = tp.rowInfo + 4*(size_t)ro;
	int iters = P.iterations;
	int tid = threadIdx.x, nt = blockDim.x;
	int nbw = W.nbodies, bo = W.bodyOff;
	int nb = s.totalBodies;
	const double *bd = tp.body + (size_t)t*8*nb;

	/* 1. adjoints of the impulses stored at the end of the step */
	for(int k = tid; k < n; k += nt){
		const cpgRow &row = rows[k];
		for(int c = 0; c < 2; c++){
			AdjScratch *sc = con_scratch(a, ro + k, c);
			adj_zero(sc->cb);
			sc->jN = 0.0; sc->jT = 0.0; sc->jB = 0.0;
			if(row.kind == 0){
				double *arb = a.arb + 4*(size_t)row.src + 2*c;
				if(c < row.count){ sc->jN = arb[0]; sc->jT = arb[1]; }
				arb[0] = 0.0; arb[1] = 0.0;
			}
		}
	}
	__syncthreads();

	/* 2. iterations in reverse */
	for(int pass = iters; pass >= 1; pass--){
		for(int l = nlev - 1; l >= 0; l--){
			for(int k = start[l] + tid; k < start[l + 1]; k += nt){
				const cpgRow &row = rows[k];
				if(row.kind != 0) continue;
				int ga = bo + row.a, gb = bo + row.b;
				bool da = (row.flags & ROW_DYN_A_) != 0, db = (row.flags & ROW_DYN_B_) != 0;
				AdjBody A = {0, 0, 0, 0, 0, 0}, B = {0, 0, 0, 0, 0, 0};
				if(da) A = load_bar(a, ga);
				if(db) B = load_bar(a, gb);
				const AdjApp *rec = (const AdjApp *)tp.app + ((size_t)(ro + k)*iters + (pass - 1))*2;
				for(int c = row.count - 1; c >= 0; c--){
					AdjCon con = make_con(s, row, c, ga, gb);
					AdjScratch *sc = con_scratch(a, ro + k, c);
					app_adjoint(con, rec[c], A, B, sc->jN, sc->jT, sc->jB, sc->cb);
				}
				if(da) store_bar(a, ga, A);
				if(db) store_bar(a, gb, B);
			}
			__syncthreads();
		}
	}

	/* 3. warm start (reads the body adjoints only), then the initial
	 * accumulators' adjoints go to their source contacts */
	for(int k = tid; k < n; k += nt){
		const cpgRow &row = rows[k];
		if(row.kind != 0) continue;
		int ga = bo + row.a, gb = bo + row.b;
		bool da = (row.flags & ROW_DYN_A_) != 0, db = (row.flags & ROW_DYN_B_) != 0;
		AdjBody A = {0, 0, 0, 0, 0, 0}, B = {0, 0, 0, 0, 0, 0};
		if(da) A = load_bar(a, ga);
		if(db) B = load_bar(a, gb);
		int src = info[4*k + 3];
		for(int c = row.count - 1; c >= 0; c--){
			AdjCon con = make_con(s, row, c, ga, gb);
			AdjScratch *sc = con_scratch(a, ro + k, c);
			if(!(row.flags & ROW_FIRST_))
				warm_adjoint(con, row.arb.c[c].jnAcc, row.arb.c[c].jtAcc, P.dt_coef, A, B, sc->jN, sc->jT, sc->cb);
			int j = ((src >> (4*c)) & 0xF) - 1;
			if(j >= 0 && j < 2){
				double *arb = a.arb + 4*(size_t)row.src + 2*j;
				arb[0] += sc->jN; arb[1] += sc->jT;
			}
		}
	}
	__syncthreads();

	/* 4. velocity integration; the bias velocities start the solve at 0 */
	for(int i = tid; i < nbw; i += nt){
		int g = bo + i;
		if(s.btype[g] != CPG_DYNAMIC) continue;
		double *b = a.body + 9*(size_t)g;
		b[3] *= P.damping; b[4] *= P.damping; b[5] *= P.damping;
		b[6] = 0.0; b[7] = 0.0; b[8] = 0.0;
	}
	__syncthreads();

	/* 5. pre-step and contact geometry, by levels */
	for(int l = nlev - 1; l >= 0; l--){
		for(int k = start[l] + tid; k < start[l + 1]; k += nt){
			const cpgRow &row = rows[k];
			if(row.kind != 0) continue;
			int ga = bo + row.a, gb = bo + row.b;
			bool da = (row.flags & ROW_DYN_A_) != 0, db = (row.flags & ROW_DYN_B_) != 0;
			double r1bar[4] = {0, 0, 0, 0}, r2bar[4] = {0, 0, 0, 0}, nbx = 0.0, nby = 0.0;
			AdjPreBar tot; adj_zero(tot);
			double uArb = 0.0, mA = 0.0, mB = 0.0;
			for(int c = 0; c < row.count && c < 2; c++){
				const cpgRowContact &rc = row.arb.c[c];
				AdjPre p;
				p.r1x = rc.r1x; p.r1y = rc.r1y; p.r2x = rc.r2x; p.r2y = rc.r2y;
				p.nx = row.arb.nx; p.ny = row.arb.ny;
				p.pAx = bd[ga]; p.pAy = bd[nb + ga]; p.pBx = bd[gb]; p.pBy = bd[nb + gb];
				p.vAx = bd[3*(size_t)nb + ga]; p.vAy = bd[4*(size_t)nb + ga]; p.wA = bd[5*(size_t)nb + ga];
				p.vBx = bd[3*(size_t)nb + gb]; p.vBy = bd[4*(size_t)nb + gb]; p.wB = bd[5*(size_t)nb + gb];
				p.minvA = s.minv[ga]; p.minvB = s.minv[gb]; p.iinvA = s.iinv[ga]; p.iinvB = s.iinv[gb];
				p.e = row.arb.e;
				p.biasCoef = P.biasCoef; p.slop = P.slop; p.dt = P.dt;
				const AdjScratch *sc = con_scratch(a, ro + k, c);
				AdjPreBar pb; adj_zero(pb);
				prestep_adjoint(p, sc->cb.nMass, sc->cb.tMass, sc->cb.bias, sc->cb.bounce, pb);
				r1bar[2*c] = sc->cb.r1x + pb.r1x; r1bar[2*c + 1] = sc->cb.r1y + pb.r1y;
				r2bar[2*c] = sc->cb.r2x + pb.r2x; r2bar[2*c + 1] = sc->cb.r2y + pb.r2y;
				nbx += sc->cb.nx + pb.nx; nby += sc->cb.ny + pb.ny;
				tot.pAx += pb.pAx; tot.pAy += pb.pAy; tot.pBx += pb.pBx; tot.pBy += pb.pBy;
				tot.vAx += pb.vAx; tot.vAy += pb.vAy; tot.wA += pb.wA;
				tot.vBx += pb.vBx; tot.vBy += pb.vBy; tot.wB += pb.wB;
				tot.e += pb.e;
				uArb += sc->cb.u;
				mA += sc->cb.minvA + pb.minvA; mB += sc->cb.minvB + pb.minvB;
			}
			/* geometry: the arbiter's shapes in the order the forward stored */
			int sa = W.shapeOff + info[4*k], sb = W.shapeOff + info[4*k + 1];
			GShape SA = tape_gshape(s, t, sa, ga, da ? 0 : -1);
			GShape SB = tape_gshape(s, t, sb, gb, db ? 1 : -1);
			GContacts g;
			geom_contacts(SA, SB, (unsigned)info[4*k + 2], g);
			double pose[6] = {0, 0, 0, 0, 0, 0};
			if(g.count == row.count) geom_adjoint(g, row.count, r1bar, r2bar, nbx, nby, pose);
			else atomicOr(&tp.cursor[3], 2);
			if(da){
				double *b = a.body + 9*(size_t)ga;
				b[0] += pose[0] + tot.pAx; b[1] += pose[1] + tot.pAy; b[2] += pose[2];
				b[3] += tot.vAx; b[4] += tot.vAy; b[5] += tot.wA;
				a.gMinv[ga] += mA;
			}
			if(db){
				double *b = a.body + 9*(size_t)gb;
				b[0] += pose[3] + tot.pBx; b[1] += pose[4] + tot.pBy; b[2] += pose[5];
				b[3] += tot.vBx; b[4] += tot.vBy; b[5] += tot.wB;
				a.gMinv[gb] += mB;
			}
			a.unit[2*(size_t)(ro + k)] = tot.e;
			a.unit[2*(size_t)(ro + k) + 1] = uArb;
		}
		__syncthreads();
	}

	/* 6. position integration: p' = p + (v + v_bias)*dt, a' = a + (w + w_bias)*dt */
	for(int i = tid; i < nbw; i += nt){
		int g = bo + i;
		if(s.btype[g] != CPG_DYNAMIC) continue;
		double *b = a.body + 9*(size_t)g;
		double dt = P.dt;
		b[3] += b[0]*dt; b[4] += b[1]*dt; b[5] += b[2]*dt;
		b[6] = b[0]*dt; b[7] = b[1]*dt; b[8] = b[2]*dt;
	}

	/* per-shape elasticity and friction, in unit order */
	if(tid == 0){
		for(int k = 0; k < n; k++){
			const cpgRow &row = rows[k];
			if(row.kind != 0) continue;
			int sa = W.shapeOff + info[4*k], sb = W.shapeOff + info[4*k + 1];
			double eb = a.unit[2*(size_t)(ro + k)], ub = a.unit[2*(size_t)(ro + k) + 1];
			a.gE[sa] += eb*s.se[sb]; a.gE[sb] += eb*s.se[sa];
			a.gU[sa] += ub*s.su[sb]; a.gU[sb] += ub*s.su[sa];
		}
	}
}

extern "C" int cpg_launch_adjoint(const cpgSet *s, const cpgAdj *a, int step, void *stream)
{
	k_adj_step<<<s->nworlds, 256, 0, (cudaStream_t)stream>>>(*s, *a, step);
	return cudaGetLastError() == cudaSuccess ? 0 : -1;
}
