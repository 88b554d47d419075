/*
 * acum_oracle.c -- CPU restatement, in plain C and FP64 throughout, of the reference's
 * periodic acoustic hot path (dilharaj/ACUM3_periodic).
 *
 * TEST INFRASTRUCTURE: this is the oracle.  Only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load it, and only as the reference the GPU results are
 * compared with (or as the timed CPU port in that leg).  The GPU product never calls into
 * it.
 *
 * Pinning: tests/test_oracle_pin.py compares every function here with the reference's
 * own sources compiled in FP64 (oracle/build_ref.sh -> oracle/_ref/libacumref_f64.so) on
 * seeded decks, and tests/test_golden.py compares it with the committed golden vectors
 * that tests/golden/make_golden.py generated from that build.
 *
 * It follows the reference algorithm step by step (serial loops, the binary-search bin
 * lookup, the backward/forward hat walks, the dB log-adds of the broadband model), not
 * the GPU formulation, so that it is an independent check of the kernels.
 *
 * Layouts (all double):
 *   raw    [surface][step][element][8]  x, y, z, Cp, A, nx, ny, nz  (a surface_*.dat row)
 *   fields [element][step][18]  x,y,z,ds | n(3),ndot(3) | V(3),Vdot(3) | P,Pdot
 *          (the per-element-step contents of Xham/Nham/Vham/PRham, variables.cu:54)
 *   obs    [observer][3]        positions after OBSscale (io.cu:123-129)
 *   pT/pL/pA [step][observer]   as main.cu:123-130
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>

#define F_X 0
#define F_DS 3
#define F_N 4
#define F_ND 7
#define F_V 10
#define F_VD 13
#define F_P 16
#define F_PD 17
#define NFIELD 18

typedef struct {
    int nsurf, ntime, nobs;
    const int* nelem;    /* elements per surface */
    double a0, rho_ref, om, dpsi, dtau; /* dpsi in radians, as after io.cu:74-75 */
    double vinf[3];
    double mref, cfd_scale;
    int periodic, lowpass;
} acumo_tonal;

/* ------------------------------------------------------------------ mathfunc.cu */

/* mathfunc.cu:132-140 -- periodic second-order central difference */
static void o_diff_periodic(const double* u, double* du, double dt, int n)
{
    du[0] = (u[1] - u[n - 1]) / (2.0 * dt);
    du[n - 1] = (u[0] - u[n - 2]) / (2.0 * dt);
    for (int k = 1; k < n - 1; k++) du[k] = (u[k + 1] - u[k - 1]) / (2.0 * dt);
}

/* mathfunc.cu:142-159 -- central interior, ends replaced by cubic extrapolation */
static void o_diff_biased(const double* u, double* du, double dt, int n)
{
    for (int k = 1; k < n - 1; k++) du[k] = (u[k + 1] - u[k - 1]) / (2.0 * dt);
    du[0] = 3 * du[1] - 3 * du[2] + du[3];
    du[n - 1] = 3 * du[n - 2] - 3 * du[n - 3] + du[n - 4];
}

/* mathfunc.cu:165-206 with is=0 -- removes the end mismatch of a series with a cubic
 * through a linearly extrapolated point before the first sample. */
static void o_make_periodic(double* f, int n)
{
    double* g = (double*)malloc(sizeof(double) * (size_t)(n + 1));
    for (int k = 0; k < n; k++) g[k + 1] = f[k];
    g[0] = g[1] - (g[2] - g[1]);
    double k2 = g[n], k1 = g[0];
    double s2 = g[n] - g[n - 1], s1 = g[1] - g[0];
    int xm = n;
    double d = k1, c = s1 - s2;
    double b = -2.0 * (s1 - s2) / xm - 3.0 * (k1 - k2) / xm / xm;
    double a = -b / xm - (s1 - s2) / xm / xm - (k1 - k2) / xm / xm / xm;
    for (int k = 0; k <= n; k++) {
        double cub = a * k * k * k + b * k * k + c * k + d;
        g[k] = g[k] - (cub - k2);
    }
    for (int k = 0; k < n; k++) f[k] = g[k + 1];
    free(g);
}

/* mathfunc.cu:208-341 -- 3-point periodic "median": the first of (left, centre) that is
 * strictly inside (min, max), else the right neighbour (ties therefore pick the right). */
static void o_median3(double* f, int n)
{
    double* out = (double*)malloc(sizeof(double) * (size_t)n);
    for (int k = 0; k < n; k++) {
        double l = f[(k + n - 1) % n], m = f[k], r = f[(k + 1) % n];
        double hi = l > m ? l : m;
        hi = hi > r ? hi : r;
        double lo = l < m ? l : m;
        lo = lo < r ? lo : r;
        if (l < hi && l > lo) out[k] = l;
        else if (m < hi && m > lo) out[k] = m;
        else out[k] = r;
    }
    memcpy(f, out, sizeof(double) * (size_t)n);
    free(out);
}

/* mathfunc.cu:350-370 -- normalised 13-tap Gaussian with sigma = (13-1)/6 */
static void o_gauss_taps(double* w, int nw)
{
    double sd = (nw - 1) / 6.0, amp = 1.0 / (sqrt(2.0 * M_PI) * sd), tot = 0.0;
    int h = (nw - 1) / 2;
    for (int j = 0; j < nw; j++) {
        double x = j - h;
        w[j] = amp * exp(-0.5 * (x * x) / sd / sd);
        tot += w[j];
    }
    for (int j = 0; j < nw; j++) w[j] = w[j] / tot;
}

/* mathfunc.cu:375-421 -- periodic convolution with the taps */
static void o_gauss_filter(double* f, const double* w, int n, int nw)
{
    double* out = (double*)malloc(sizeof(double) * (size_t)n);
    int h = (nw - 1) / 2;
    for (int k = 0; k < n; k++) {
        double s = 0.0;
        for (int j = 0; j < nw; j++) {
            int q = k + j - h;
            if (q < 0) q += n;
            else if (q > n - 1) q -= n;
            s += w[j] * f[q];
        }
        out[k] = s;
    }
    memcpy(f, out, sizeof(double) * (size_t)n);
    free(out);
}

void acumo_make_periodic(double* f, int n) { o_make_periodic(f, n); }
void acumo_lowpass(double* f, int n)
{
    double w[13];
    o_gauss_taps(w, 13);
    for (int p = 0; p < 2; p++) {
        o_median3(f, n);
        o_gauss_filter(f, w, n, 13);
    }
}
void acumo_differentiate(const double* u, double* du, double dt, int n, int biased)
{
    if (biased) o_diff_biased(u, du, dt, n);
    else o_diff_periodic(u, du, dt, n);
}

/* ------------------------------------------------------------ preprocess.cu */

/* preprocess.cu:228-413 (preprocess_imper): scaling, make_periodic + optional lowpass on
 * the pressure, then d/dtau of P, n, x and of the resulting velocity. */
int acumo_preprocess(const acumo_tonal* p, const double* raw, double* fields)
{
    int nt = p->ntime;
    double w[13];
    o_gauss_taps(w, 13);
    double* s = (double*)malloc(sizeof(double) * (size_t)nt * 8);
    double* d = (double*)malloc(sizeof(double) * (size_t)nt * 8);
    double pscale = 0.5 * p->rho_ref * (p->mref * p->mref) * (p->a0 * p->a0);
    size_t rbase = 0;
    long ebase = 0;
    for (int is = 0; is < p->nsurf; is++) {
        int ne = p->nelem[is];
        for (int e = 0; e < ne; e++) {
            /* series of this element: x,y,z,P,nx,ny,nz (column-major into s) */
            double* X = s;
            double* Y = s + nt;
            double* Z = s + 2 * nt;
            double* P = s + 3 * nt;
            double* NX = s + 4 * nt;
            double* NY = s + 5 * nt;
            double* NZ = s + 6 * nt;
            double* out = fields + (size_t)(ebase + e) * nt * NFIELD;
            for (int k = 0; k < nt; k++) {
                const double* r = raw + rbase + ((size_t)k * ne + e) * 8;
                X[k] = r[0] * p->cfd_scale;
                Y[k] = r[1] * p->cfd_scale;
                Z[k] = r[2] * p->cfd_scale;
                P[k] = r[3] * pscale;
                NX[k] = r[5];
                NY[k] = r[6];
                NZ[k] = r[7];
                out[(size_t)k * NFIELD + F_DS] = r[4] * p->cfd_scale * p->cfd_scale;
            }
            o_make_periodic(P, nt);
            if (p->lowpass == 1) {
                for (int q = 0; q < 2; q++) {
                    o_median3(P, nt);
                    o_gauss_filter(P, w, nt, 13);
                }
            }
            double* PD = d;
            double* NDX = d + nt;
            double* NDY = d + 2 * nt;
            double* NDZ = d + 3 * nt;
            double* VX = d + 4 * nt;
            double* VY = d + 5 * nt;
            double* VZ = d + 6 * nt;
            if (p->periodic == 1) o_diff_periodic(P, PD, p->dtau, nt);
            else o_diff_biased(P, PD, p->dtau, nt);
            o_diff_periodic(NX, NDX, p->dtau, nt);
            o_diff_periodic(NY, NDY, p->dtau, nt);
            o_diff_periodic(NZ, NDZ, p->dtau, nt);
            o_diff_periodic(X, VX, p->dtau, nt);
            o_diff_periodic(Y, VY, p->dtau, nt);
            o_diff_periodic(Z, VZ, p->dtau, nt);
            double* acc = (double*)malloc(sizeof(double) * (size_t)nt * 3);
            o_diff_periodic(VX, acc, p->dtau, nt);
            o_diff_periodic(VY, acc + nt, p->dtau, nt);
            o_diff_periodic(VZ, acc + 2 * nt, p->dtau, nt);
            for (int k = 0; k < nt; k++) {
                double* o = out + (size_t)k * NFIELD;
                o[F_X + 0] = X[k]; o[F_X + 1] = Y[k]; o[F_X + 2] = Z[k];
                o[F_N + 0] = NX[k]; o[F_N + 1] = NY[k]; o[F_N + 2] = NZ[k];
                o[F_ND + 0] = NDX[k]; o[F_ND + 1] = NDY[k]; o[F_ND + 2] = NDZ[k];
                o[F_V + 0] = VX[k]; o[F_V + 1] = VY[k]; o[F_V + 2] = VZ[k];
                o[F_VD + 0] = acc[k]; o[F_VD + 1] = acc[nt + k]; o[F_VD + 2] = acc[2 * nt + k];
                o[F_P] = P[k];
                o[F_PD] = PD[k];
            }
            free(acc);
        }
        rbase += (size_t)nt * ne * 8;
        ebase += ne;
    }
    free(s);
    free(d);
    return 0;
}

/* preprocess.cu:8-226 (preprocess_per), the permeable surfaces' preprocessing, in place
 * on the elements of all surfaces stacked [element][step][k]: X (x, y, z, ds), N (n,
 * ndot), V (V, Vdot), U (u, udot), PR (P, Pdot, rho, rhodot); scal = dTau, a0, rhoRef,
 * Mref, CFDscale.  Scaling (preprocess.cu:50-68, left to right as written there), the
 * optional low-pass of rho, u, P (113-137, no make_periodic), their derivatives periodic
 * or end-biased (150-163), ndot periodic (166-168), V = dx/dtau and Vdot = dV/dtau
 * periodic (172-180). */
int acumo_preprocess_per(int E, int nt, const double* scal, int periodic, int lowpass, double* X, double* N,
                         double* V, double* U, double* PR)
{
    const double dt = scal[0], a0 = scal[1], rho_ref = scal[2], mref = scal[3], cfd = scal[4];
    const size_t n = (size_t)E * nt;
    for (size_t i = 0; i < n; i++) {
        double* x = X + 4 * i;
        x[0] = x[0] * cfd;
        x[1] = x[1] * cfd;
        x[2] = x[2] * cfd;
        x[3] = x[3] * cfd * cfd;
        PR[4 * i + 2] = PR[4 * i + 2] * rho_ref;
        U[6 * i + 0] = U[6 * i + 0] * a0;
        U[6 * i + 1] = U[6 * i + 1] * a0;
        U[6 * i + 2] = U[6 * i + 2] * a0;
        PR[4 * i + 0] = PR[4 * i + 0] * 0.5 * rho_ref * pow(mref, 2) * pow(a0, 2);
    }
    double w[13];
    o_gauss_taps(w, 13);
    double* f = (double*)malloc(sizeof(double) * (size_t)nt);
    double* d = (double*)malloc(sizeof(double) * (size_t)nt);
    double* g = (double*)malloc(sizeof(double) * (size_t)nt);
    for (int e = 0; e < E; e++) {
        /* flow series in the reference's order v1..v5: rho, u, v, w, P */
        double* base[5] = {PR + 2, U + 0, U + 1, U + 2, PR + 0};
        double* dbase[5] = {PR + 3, U + 3, U + 4, U + 5, PR + 1};
        const int stride[5] = {4, 6, 6, 6, 4};
        for (int v = 0; v < 5; v++) {
            double* col = base[v] + (size_t)e * nt * stride[v];
            double* dcol = dbase[v] + (size_t)e * nt * stride[v];
            for (int k = 0; k < nt; k++) f[k] = col[(size_t)k * stride[v]];
            if (lowpass == 1)
                for (int q = 0; q < 2; q++) {
                    o_median3(f, nt);
                    o_gauss_filter(f, w, nt, 13);
                }
            if (periodic == 1) o_diff_periodic(f, d, dt, nt);
            else o_diff_biased(f, d, dt, nt);
            for (int k = 0; k < nt; k++) {
                col[(size_t)k * stride[v]] = f[k];
                dcol[(size_t)k * stride[v]] = d[k];
            }
        }
        double* ne = N + (size_t)e * nt * 6;
        double* xe = X + (size_t)e * nt * 4;
        double* ve = V + (size_t)e * nt * 6;
        for (int c = 0; c < 3; c++) {
            for (int k = 0; k < nt; k++) f[k] = ne[(size_t)k * 6 + c];
            o_diff_periodic(f, d, dt, nt);
            for (int k = 0; k < nt; k++) ne[(size_t)k * 6 + 3 + c] = d[k];
            for (int k = 0; k < nt; k++) f[k] = xe[(size_t)k * 4 + c];
            o_diff_periodic(f, d, dt, nt);
            o_diff_periodic(d, g, dt, nt);
            for (int k = 0; k < nt; k++) {
                ve[(size_t)k * 6 + c] = d[k];
                ve[(size_t)k * 6 + 3 + c] = g[k];
            }
        }
    }
    free(f);
    free(d);
    free(g);
    return 0;
}

/* ------------------------------------------------------------------ core.cu */

/* core.cu:261-279 -- convected retarded distance: the smaller positive root of
 * (|v|^2-a0^2) t^2 - 2 (d.v) t + |d|^2 = 0, returned as a0 t. */
static double o_retarded_distance(const double* src, const double* obs, const double* v, double a0, int* bad)
{
    double dx = obs[0] - src[0], dy = obs[1] - src[1], dz = obs[2] - src[2];
    double qa = v[0] * v[0] + v[1] * v[1] + v[2] * v[2] - a0 * a0;
    double qb = -2 * (dx * v[0] + dy * v[1] + dz * v[2]);
    double qc = dx * dx + dy * dy + dz * dz;
    double disc = qb * qb - 4 * qa * qc;
    if (disc < 0.0) *bad += 1;
    double t = (-qb - sqrt(disc)) / (2.0 * qa);
    if (t < 0.0) t = (-qb + sqrt(disc)) / (2.0 * qa);
    return t * a0;
}

/* core.cu:325-355 -- largest index i in [imin, imax) with A[i] <= key, or -1 */
static int o_bin_search(const double* A, double key, int imin, int imax)
{
    int n = imax;
    for (;;) {
        int mid = (imin + imax) / 2;
        if (key < A[mid]) imax = mid;
        else imin = mid;
        if (imin + 1 >= imax) break;
    }
    return (imin <= n && A[imin] <= key) ? imin : -1;
}

typedef struct {
    const acumo_tonal* p;
    const double* fields;
    const double* obs;
    int o0, o1; /* observer range of this shard */
    double *pT, *pL, *pA;
    int nobs_out;
    int obs_base;
    int bad;
} tonal_job;

/* core.cu:18-259 run serially for one observer shard.  The loop nest is kept in the
 * reference's order (step, observer, surface, element) so the FP64 sums are formed in
 * the same order as the reference's FP64 build run on one host thread. */
static void* o_tonal_shard(void* arg)
{
    tonal_job* J = (tonal_job*)arg;
    const acumo_tonal* p = J->p;
    int nt = p->ntime;
    double a0 = p->a0, lpi = nt * p->dpsi;
    double* tb = (double*)malloc(sizeof(double) * (size_t)nt);
    for (int t = 0; t < nt; t++) tb[t] = t * p->dpsi;
    double D1 = 1.0 / (4.0 * M_PI * a0);
    for (int itau = 0; itau < nt; itau++) {
        for (int io = J->o0; io < J->o1; io++) {
            const double* ob = J->obs + 3 * io;
            long ebase = 0;
            for (int is = 0; is < p->nsurf; is++) {
                for (int e = 0; e < p->nelem[is]; e++) {
                    const double* row = J->fields + ((size_t)(ebase + e) * nt) * NFIELD;
                    const double* f = row + (size_t)itau * NFIELD;
                    double tau = itau * p->dtau;
                    double ds = f[F_DS], P = f[F_P], Pd = f[F_PD];
                    const double* V = f + F_V;
                    const double* Vd = f + F_VD;
                    const double* N = f + F_N;
                    const double* Nd = f + F_ND;
                    double r = o_retarded_distance(f + F_X, ob, p->vinf, a0, &J->bad);
                    double rh[3];
                    for (int i = 0; i < 3; i++) rh[i] = (ob[i] - f[F_X + i] - p->vinf[i] * r / a0) / r;
                    double Mr = (V[0] * rh[0] + V[1] * rh[1] + V[2] * rh[2]) / a0;
                    double M = sqrt(V[0] * V[0] + V[1] * V[1] + V[2] * V[2]) / a0;
                    double Mdr = (Vd[0] * rh[0] + Vd[1] * rh[1] + Vd[2] * rh[2]) / a0;
                    double om = 1.0 - Mr;
                    double T1 = D1 / (r * (om * om));
                    double T2 = T1 / om, T3 = T1 / r, T4 = T3 / om;
                    /* thickness: U = V on the surface and the normal-velocity rates are
                     * forced to zero (core.cu:105-128) */
                    double Vn = V[0] * N[0] + V[1] * N[1] + V[2] * N[2];
                    double Man = p->rho_ref * Vn;
                    double pth = a0 * Man * (Mr - M * M) * T4 * a0 * ds + Man * Mdr * T2 * a0 * ds;
                    /* loading (core.cu:130-141); the momentum terms are identically 0
                     * because U - V = 0 (core.cu:143-152) */
                    double L[3], Ld[3];
                    for (int i = 0; i < 3; i++) {
                        L[i] = P * N[i];
                        Ld[i] = Pd * N[i] + P * Nd[i];
                    }
                    double Ldr = Ld[0] * rh[0] + Ld[1] * rh[1] + Ld[2] * rh[2];
                    double Lr = L[0] * rh[0] + L[1] * rh[1] + L[2] * rh[2];
                    double Lm = (L[0] * V[0] + L[1] * V[1] + L[2] * V[2]) / a0;
                    double far = Ldr * T1 * ds + Lr * Mdr * T2 * ds;
                    double nea = (Lr - Lm) * T3 * a0 * ds + Lr * (Mr - M * M) * T4 * a0 * ds;
                    double pld = nea + far;
                    /* core.cu:156 and 290-322: observer time and its periodic bin */
                    double tc = (tau + r / a0) * p->om;
                    int npi = (int)floor((lpi + tb[0] - tc) / lpi);
                    int ipts = o_bin_search(tb, tc + npi * lpi, 0, nt);
                    if (ipts < 0) { J->bad += 1; ipts = 0; }
                    /* core.cu:173-194: neighbour observer times with the periodic wrap */
                    int mm = itau > 0 ? itau - 1 : nt - 1, nm = itau > 0 ? 0 : 1;
                    int mp = itau < nt - 1 ? itau + 1 : 0, np = itau < nt - 1 ? 0 : 1;
                    double rm = o_retarded_distance(row + (size_t)mm * NFIELD + F_X, ob, p->vinf, a0, &J->bad);
                    double tm = ((mm * p->dtau) + rm / a0) * p->om - nm * lpi;
                    double rp = o_retarded_distance(row + (size_t)mp * NFIELD + F_X, ob, p->vinf, a0, &J->bad);
                    double tp = ((mp * p->dtau) + rp / a0) * p->om + np * lpi;
                    /* core.cu:196-231: backward and forward hat deposits */
                    int ib = ipts;
                    double tbin = tb[ib];
                    while (tbin > tm + npi * lpi) {
                        double w = (tm + npi * lpi - tbin) / (tm - tc);
                        size_t q = (size_t)ib * J->nobs_out + (io - J->obs_base);
                        J->pT[q] += pth * w;
                        J->pL[q] += pld * w;
                        J->pA[q] += (pth + pld) * w;
                        tbin -= p->dpsi;
                        ib -= 1;
                        if (ib < 0) ib = nt - 1;
                    }
                    int ifw = ipts < nt - 1 ? ipts + 1 : 0;
                    tbin = tb[ifw];
                    if (ifw == 0) tbin += lpi;
                    while (tbin < tp + npi * lpi) {
                        double w = (tp + npi * lpi - tbin) / (tp - tc);
                        size_t q = (size_t)ifw * J->nobs_out + (io - J->obs_base);
                        J->pT[q] += pth * w;
                        J->pL[q] += pld * w;
                        J->pA[q] += (pth + pld) * w;
                        tbin += p->dpsi;
                        ifw += 1;
                        if (ifw > nt - 1) ifw = 0;
                    }
                }
                ebase += p->nelem[is];
            }
        }
    }
    free(tb);
    return NULL;
}

/* Accumulates into pT/pL/pA ([step][nob], as the reference kernel does) for observers
 * [obs0, obs0+nob), using up to nthreads host threads over observer shards.
 * Returns the number of invalid-geometry events (negative discriminant or failed bin
 * search, both of which the reference only prints). */
int acumo_tonal_run(const acumo_tonal* p, const double* fields, const double* obs, int obs0, int nob,
                    double* pT, double* pL, double* pA, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > nob) nthreads = nob;
    tonal_job* jobs = (tonal_job*)calloc((size_t)nthreads, sizeof(tonal_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int k = 0; k < nthreads; k++) {
        jobs[k].p = p;
        jobs[k].fields = fields;
        jobs[k].obs = obs;
        jobs[k].o0 = obs0 + (int)((long)nob * k / nthreads);
        jobs[k].o1 = obs0 + (int)((long)nob * (k + 1) / nthreads);
        jobs[k].pT = pT;
        jobs[k].pL = pL;
        jobs[k].pA = pA;
        jobs[k].nobs_out = nob;
        jobs[k].obs_base = obs0;
    }
    for (int k = 1; k < nthreads; k++) pthread_create(&th[k], NULL, o_tonal_shard, &jobs[k]);
    o_tonal_shard(&jobs[0]);
    int bad = jobs[0].bad;
    for (int k = 1; k < nthreads; k++) {
        pthread_join(th[k], NULL);
        bad += jobs[k].bad;
    }
    free(jobs);
    free(th);
    return bad;
}

/* ============================================================ broadband (BPM) */

typedef struct {
    int nsurf, ntime, nobs, nf, t_del;
    double dtau, a0, vinf[3];
    const double* ff;           /* [nf] band centres (io.cu:693-699) */
    /* per BB surface (io.cu:357-414) */
    const double *span, *omega, *psi_offset, *rotate, *translate; /* rotate/translate [3] each */
    const int *ccw, *trip, *nsect;
    /* BB_surface data, surfaces concatenated: xyzcR [sum nsect][4]; bbdata [surf][step][sect][7]
     * with cn,cc already divided by (r/R)^2 as io.cu:509-512 does at read time */
    const double *xyzcR, *bbdata;
    /* tables, surfaces concatenated: sizes per surface, axes, data [sect][mach][re][aoa][7] */
    const int *nsect_t, *naoa_t, *nmach_t, *nre_t;
    const double *sect_t, *aoa_t, *mach_t, *re_t, *bbdata_t;
    int aa_mode; /* 0: convected time with aa = a0^2-|v|^2 (corrected); 1: aa = 0 */
} acumo_bpm;

/* bb_utils.cu:6-88 -- BPM spectral shape curves A_min, A_max, B_min, B_max */
static double o_amin(double a)
{
    if (a < 0.204) return sqrt(67.552 - 886.788 * (a * a)) - 8.219;
    if (a > 0.244) return -142.795 * (a * a * a) + 103.656 * (a * a) - 57.757 * a + 6.006;
    return -32.665 * a + 3.981;
}
static double o_amax(double a)
{
    if (a < 0.13) return sqrt(67.552 - 886.788 * (a * a)) - 8.219;
    if (a > 0.321) return -4.669 * (a * a * a) + 3.491 * (a * a) - 16.699 * a + 1.149;
    return -15.901 * a + 1.098;
}
static double o_bmin(double b)
{
    if (b < 0.13) return sqrt(16.888 - 886.788 * (b * b)) - 4.109;
    if (b > 0.145) return -817.810 * (b * b * b) + 355.21 * (b * b) - 135.024 * b + 10.619;
    return -83.607 * b + 8.138;
}
static double o_bmax(double b)
{
    if (b < 0.1) return sqrt(16.888 - 886.788 * (b * b)) - 4.109;
    if (b > 0.187) return -80.541 * (b * b * b) + 44.174 * (b * b) - 39.381 * b + 2.344;
    return -31.313 * b + 1.854;
}

/* bb_utils.cu:90-121 -- bluntness spectrum shape G5 */
static double o_g5(double h, double eta)
{
    double mu, m;
    if (h <= 0.25) mu = 0.1211;
    else if (h <= 0.62) mu = -0.2175 * h + 0.1755;
    else if (h < 1.15) mu = -0.0308 * h + 0.0596;
    else mu = 0.0242;
    if (h <= 0.02) m = 0.0;
    else if (h < 0.5) m = 68.724 * h - 1.35;
    else if (h <= 0.62) m = 308.475 * h - 121.23;
    else if (h <= 1.15) m = 224.811 * h - 69.354;
    else if (h < 1.2) m = 1583.28 * h - 1631.592;
    else m = 268.344;
    if (m < 0.0) m = 0.0;
    double eta0 = -sqrt((m * m * (mu * mu * mu * mu)) / (6.25 + m * m * mu * mu));
    double k = 2.5 * sqrt(1.0 - (eta0 / mu) * (eta0 / mu)) - 2.5 - m * eta0;
    if (eta <= eta0) return m * eta + k;
    if (eta <= 0.0) return 2.5 * sqrt(1.0 - (eta / mu) * (eta / mu)) - 2.5;
    if (eta <= 0.03616) return sqrt(1.5625 - 1194.99 * (eta * eta)) - 1.25;
    return -155.543 * eta + 4.375;
}

void acumo_bb_curve(int which, const double* x, double* y, int n)
{
    for (int i = 0; i < n; i++)
        y[i] = which == 0 ? o_amin(x[i]) : which == 1 ? o_amax(x[i]) : which == 2 ? o_bmin(x[i]) : o_bmax(x[i]);
}
double acumo_g5comp(double h, double eta) { return o_g5(h, eta); }

static double db_add(double a, double b) { return 10.0 * log10(pow(10.0, a / 10.0) + pow(10.0, b / 10.0)); }

/* bb_core.cu:591-1043 -- BPM sub-models for one (observer, section, step); log-adds the
 * seven component levels of every band into out[nf][7] as the reference does. */
void acumo_bpm_core(double rpn, double th, double ph, double c, double ls, double alpha, double u, double nu,
                    double a0, int trip, double del_s, double del_p, double dis_s, double dis_p, int isect, int nsect,
                    const double* ff, int nf, double R, double* out)
{
    if (del_s < 0.0) del_s = 1.0e-10;
    if (del_p < 0.0) del_p = 1.0e-10;
    if (dis_p < 0.0) dis_p = 1.0e-10;
    if (dis_s < 0.0) dis_s = 1.0e-10;
    u = fabs(u);
    double M = u / a0, rc = u * c / nu, mc = 0.6 * u / a0;
    if (th == 0) th = 1e-10;
    if (ph == 0) ph = 1e-10;
    /* high-frequency and low-frequency directivities (bb_core.cu:620-624) */
    double sh = sin(th / 2.0), sp = sin(ph), ct = cos(th);
    double dh = (2.0 * (sh * sh) * (sp * sp)) / ((1.0 + M * ct) * ((1.0 + (M - mc) * ct) * (1.0 + (M - mc) * ct)));
    double st = sin(th), q1 = 1.0 + M * ct;
    double dl = ((st * st) * (sp * sp)) / (q1 * q1 * q1 * q1);

    /* --- TBL-TE (bb_core.cu:630-859) --- */
    double rdp = u * dis_p / nu;
    double st1 = 0.02 * pow(M, -0.6), st2;
    if (alpha < 1.33) st2 = st1;
    else if (alpha > 12.5) st2 = st1 * 4.72;
    else st2 = st1 * pow(10.0, 0.0054 * ((alpha - 1.33) * (alpha - 1.33)));
    double a0r;
    if (rc < 9.52e4) a0r = 0.57;
    else if (rc > 8.57e5) a0r = 1.13;
    else a0r = (-9.57e-13) * ((rc - 8.57e5) * (rc - 8.57e5)) + 1.13;
    double ar = (-20.0 - o_amin(a0r)) / (o_amax(a0r) - o_amin(a0r));
    double b0r;
    if (rc < 9.52e4) b0r = 0.3;
    else if (rc > 8.57e5) b0r = 0.56;
    else b0r = (-4.48e-13) * ((rc - 8.57e5) * (rc - 8.57e5)) + 0.56;
    double br = (-20.0 - o_bmin(b0r)) / (o_bmax(b0r) - o_bmin(b0r));
    double k1;
    if (rc < 2.47e5) k1 = -4.31 * log10(rc) + 156.3;
    else if (rc > 8.0e5) k1 = 128.5;
    else k1 = -9.0 * log10(rc) + 181.6;
    double dk1 = rdp <= 5000 ? alpha * (1.43 * log10(rdp) - 5.29) : 0.0;
    double gam = 27.094 * M + 3.31, gam0 = 23.43 * M + 4.651;
    double bet = 72.65 * M + 10.74, bet0 = -34.19 * M - 13.82;
    double k2;
    if (alpha < gam0 - gam) k2 = k1 - 1000.0;
    else if (alpha > gam0 + gam) k2 = k1 - 12.0;
    else k2 = k1 + sqrt(bet * bet - (bet / gam) * (bet / gam) * ((alpha - gam0) * (alpha - gam0))) + bet0;
    int stall = (alpha >= gam0 || alpha > 12.5);
    double k2s = 0.0, ars = 0.0;
    if (stall) {
        double rcn = 3.0 * rc, a0n;
        if (rcn < 9.52e4) a0n = 0.57;
        else if (rcn > 8.57e5) a0n = 1.13;
        else a0n = -9.57e-13 * ((rcn - 8.57e5) * (rcn - 8.57e5)) + 1.13;
        double k1n;
        if (rcn < 2.47e5) k1n = -4.31 * log10(rcn) + 156.3;
        else if (rcn > 8e5) k1n = 128.5;
        else k1n = -9.0 * log10(rcn) + 181.6;
        if (alpha < gam0 - gam) k2s = k1n - 1000.0;
        else if (alpha > gam0 + gam) k2s = k1n - 12.0;
        else k2s = k1n + sqrt(bet * bet - ((bet / gam) * (bet / gam)) * ((alpha - gam0) * (alpha - gam0))) + bet0;
        ars = (-20.0 - o_amin(a0n)) / (o_amax(a0n) - o_amin(a0n));
    }
    double m5 = pow(M, 5);
    double lvl_p = 10.0 * log10((dis_p * m5 * ls * dh) / (rpn * rpn));
    double lvl_s = 10.0 * log10((dis_s * m5 * ls * dh) / (rpn * rpn));
    double lvl_al = 10.0 * log10((dis_s * m5 * ls * dl) / (rpn * rpn));
    for (int i = 0; i < nf; i++) {
        double sts = ff[i] * dis_s / u, stp = ff[i] * dis_p / u;
        double as = fabs(log10(sts / st1)), ap = fabs(log10(stp / st1));
        double aas = o_amin(as) + ar * (o_amax(as) - o_amin(as));
        double aap = o_amin(ap) + ar * (o_amax(ap) - o_amin(ap));
        double spl_p = lvl_p + aap + (k1 - 3.0) + dk1;
        double spl_s = lvl_s + aas + (k1 - 3.0);
        double spl_a;
        if (stall) {
            double an = fabs(log10(sts / st2));
            spl_a = lvl_al + (o_amin(an) + ars * (o_amax(an) - o_amin(an))) + k2s;
        } else {
            double b = fabs(log10(sts / st2));
            spl_a = lvl_s + (o_bmin(b) + br * (o_bmax(b) - o_bmin(b))) + k2;
        }
        if (spl_a < -100) spl_a = -100.0;
        if (spl_s < -100) spl_s = -100.0;
        if (spl_p < -100) spl_p = -100.0;
        double* o = out + 7 * i;
        o[1] = db_add(o[1], spl_a);
        o[2] = db_add(o[2], spl_s);
        o[3] = db_add(o[3], spl_p);
        o[0] = 10.0 * log10(pow(10.0, o[0] / 10.0) + pow(10.0, spl_a / 10.0) + pow(10.0, spl_p / 10.0) +
                            pow(10.0, spl_s / 10.0));
    }

    /* --- LBL-VS, untripped sections only (bb_core.cu:863-915) --- */
    if (trip == 0) {
        double stl;
        if (rc < 1.3e5) stl = 0.18;
        else if (rc > 1.3e5 && rc <= 4e5) stl = 0.001756 * pow(rc, 0.3931);
        else stl = 0.28;
        double stpk = pow(10, (-0.04 * alpha)) * stl;
        double rc0 = alpha <= 3.0 ? pow(10, (0.215 * alpha + 4.978)) : pow(10, (0.120 * alpha + 5.263));
        double d = rc / rc0, g2;
        if (d <= 0.3237) g2 = 77.852 * log10(d) + 15.328;
        else if (d <= 0.5689) g2 = 65.188 * log10(d) + 9.125;
        else if (d <= 1.7579) g2 = -114.052 * (log10(d) * log10(d));
        else if (d <= 3.0889) g2 = -65.188 * log10(d) + 9.125;
        else g2 = -77.852 * log10(d) + 15.328;
        double g3 = 171.04 - 3.03 * alpha;
        double scal = 10.0 * log10(del_p * m5 * dh * ls / (rpn * rpn));
        for (int i = 0; i < nf; i++) {
            double e = (ff[i] * del_p / u) / stpk, g1, le = log10(e);
            if (e <= 0.5974) g1 = 39.8 * le - 11.12;
            else if (e <= 0.8545) g1 = 98.409 * le + 2.0;
            else if (e <= 1.17) g1 = -5.076 + sqrt(2.484 - 506.25 * (le * le));
            else if (e <= 1.674) g1 = -98.409 * le + 2.0;
            else g1 = -39.80 * le - 11.12;
            double lam = g1 + g2 + g3 + scal;
            out[7 * i + 4] = db_add(out[7 * i + 4], lam);
            out[7 * i + 0] = db_add(out[7 * i + 0], lam);
        }
    }

    /* --- TEB-VS with h = 0.5 mm, psi = 14 deg (bb_core.cu:917-971) --- */
    {
        double h = 0.0005, psi = 14.0;
        double hd = h / ((dis_s + dis_p) / 2.0), dh_ = 1.0 / hd;
        double aterm = 0.212 - 0.0045 * psi, stpeak;
        if (hd >= 0.2) stpeak = aterm / (1.0 + 0.235 * dh_ - 0.0132 * (dh_ * dh_));
        else stpeak = 0.1 * hd + 0.095 - 0.00243 * psi;
        double g4 = hd <= 5.0 ? 17.5 * log10(hd) + 157.5 - 1.114 * psi : 169.7 - 1.114 * psi;
        double hdp = 6.724 * (hd * hd) - 4.019 * hd + 1.107;
        double scal = 10.0 * log10(pow(M, 5.5) * h * dh * ls / (rpn * rpn));
        for (int i = 0; i < nf; i++) {
            double eta = log10((ff[i] * h / u) / stpeak);
            double g514 = o_g5(hd, eta), g50 = o_g5(hdp, eta);
            double g5 = g50 + 0.0714 * psi * (g514 - g50);
            if (g5 > 0) g5 = 0.0;
            double f4 = o_g5(0.25, eta);
            if (g5 > f4) g5 = f4;
            double bl = g4 + g5 + scal;
            out[7 * i + 5] = db_add(out[7 * i + 5], bl);
            out[7 * i + 0] = db_add(out[7 * i + 0], bl);
        }
    }

    /* --- tip vortex, last section only (bb_core.cu:975-1039) --- */
    if (isect == nsect - 1) {
        static const double ar0[6] = {2.0, 2.67, 4.0, 6.0, 12.0, 24.0};
        static const double rat0[6] = {0.54, 0.62, 0.71, 0.79, 0.89, 0.95};
        double AR = R / c, rat;
        if (AR < ar0[0]) rat = rat0[0];
        else if (AR > ar0[5]) rat = rat0[5];
        else {
            int kk = 0;
            while (kk < 6 && !(AR < ar0[kk])) kk++;
            rat = rat0[kk - 1] * (ar0[kk] - AR) / (ar0[kk] - ar0[kk - 1]) +
                  rat0[kk] * (AR - ar0[kk - 1]) / (ar0[kk] - ar0[kk - 1]);
        }
        double at = alpha * rat;
        double tl = fabs(at) <= 2.0 ? (0.023 + 0.0169 * at) * c : (0.0378 + 0.0095 * at) * c;
        double mm = (1.0 + 0.036 * at) * M, um = mm * a0;
        double term = M * M * (mm * mm * mm) * (tl * tl) * dh / (rpn * rpn);
        if (!(term > 2.2204460492503131e-16)) term = 2.2204460492503131e-16;
        double scal = 10.0 * log10(term);
        for (int i = 0; i < nf; i++) {
            double lg = log10(ff[i] * tl / um) + 0.3;
            double tip = 126.0 - 30.5 * (lg * lg) + scal;
            out[7 * i + 6] = db_add(out[7 * i + 6], tip);
            out[7 * i + 0] = db_add(out[7 * i + 0], tip);
        }
    }
}


/* bb_utils.cu:124-168 -- trilinear (section x Mach x Re) lookup of table column `col` at
 * AoA index `ia`; a weight of 0.5 where a bracket collapses onto one entry. */
typedef struct {
    const double *sect, *aoa, *mach, *re, *data; /* data [sect][mach][re][aoa][7] */
    int ns, na, nm, nr;
} o_table;

static double o_table_lookup(const o_table* T, double rr, double mach, double re, const int* br, int col, int ia)
{
    int is1 = br[0], is2 = br[1], im1 = br[2], im2 = br[3], ir1 = br[4], ir2 = br[5];
    double ws = is1 == is2 ? 0.5 : (rr - T->sect[is1]) / (T->sect[is2] - T->sect[is1]);
    double wm = im1 == im2 ? 0.5 : (mach - T->mach[im1]) / (T->mach[im2] - T->mach[im1]);
    double wr = ir1 == ir2 ? 0.5 : (re - T->re[ir1]) / (T->re[ir2] - T->re[ir1]);
#define TIDX(s, m, r) (((((size_t)(s) * T->nm + (m)) * T->nr + (r)) * T->na + ia) * 7 + col)
    double F1 = (1 - ws) * T->data[TIDX(is1, im1, ir1)] + ws * T->data[TIDX(is2, im1, ir1)];
    double F2 = (1 - ws) * T->data[TIDX(is1, im2, ir1)] + ws * T->data[TIDX(is2, im2, ir1)];
    double F3 = (1 - ws) * T->data[TIDX(is1, im1, ir2)] + ws * T->data[TIDX(is2, im1, ir2)];
    double F4 = (1 - ws) * T->data[TIDX(is1, im2, ir2)] + ws * T->data[TIDX(is2, im2, ir2)];
#undef TIDX
    return (1 - wm) * (1 - wr) * F1 + wm * (1 - wr) * F2 + (1 - wm) * wr * F3 + wm * wr * F4;
}

/* number of leading entries of a[] that do not exceed x (bb_core.cu:208-228) */
static int o_count_le(const double* a, int n, double x)
{
    int k = 0;
    while (k < n && !(x < a[k])) k++;
    return k;
}

/* bracket indices (is1,is2,im1,im2,ir1,ir2) as bb_core.cu:208-234 */
static void o_brackets(const o_table* T, double rr, double mach, double re, int* br)
{
    int is2 = o_count_le(T->sect, T->ns, rr), im2 = o_count_le(T->mach, T->nm, mach),
        ir2 = o_count_le(T->re, T->nr, re);
    br[0] = is2 - 1 > 0 ? is2 - 1 : 0;
    br[1] = is2 < T->ns - 1 ? is2 : T->ns - 1;
    br[2] = im2 - 1 > 0 ? im2 - 1 : 0;
    br[3] = im2 < T->nm - 1 ? im2 : T->nm - 1;
    br[4] = ir2 - 1 > 0 ? ir2 - 1 : 0;
    br[5] = ir2 < T->nr - 1 ? ir2 : T->nr - 1;
}

typedef struct {
    double *xyz, *xyzt;                /* [sect][step][3] */
    double *u, *alpha, *cla;           /* [sect][step] */
    double *bl;                        /* [sect][step][4] */
} o_bbsurf;

/* Per-(section, step) part of findBBnoise (bb_core.cu:60-444): blade kinematics, chordwise
 * flow speed, table lookups, the fixed-point effective angle of attack and the boundary
 * layer thicknesses. */
static void o_bpm_surface_prep(const acumo_bpm* B, int is, const double* geo, const double* bbd, const o_table* T,
                               o_bbsurf* S)
{
    int ns = B->nsect[is], nt = B->ntime;
    double nu = 0.0000181206 / 1.22500;
    double span = B->span[is];
    double thx = B->rotate[3 * is] * M_PI / 180, thy = B->rotate[3 * is + 1] * M_PI / 180,
           thz = B->rotate[3 * is + 2] * M_PI / 180;
    const double* tr = B->translate + 3 * is;
    int i75 = (int)round(ns * 0.75);
    double* cl = (double*)malloc(sizeof(double) * (size_t)(T->na > 0 ? T->na : 1));
    for (int k = 0; k < ns; k++) {
        double c = geo[4 * k + 3] * span;
        for (int t = 0; t < nt; t++) {
            double q[3] = {geo[4 * k] * span, geo[4 * i75 + 1] * span, geo[4 * i75 + 2] * span};
            if (B->ccw[is] == 0) q[1] = -q[1];
            double psi = (B->dtau * t * B->omega[is] + B->psi_offset[is] * M_PI / 180);
            if (B->ccw[is] == 0) psi = -psi;
            double th = bbd[((size_t)t * ns + k) * 7 + 6] * M_PI / 180;
            double e[3] = {q[0], B->ccw[is] == 1 ? q[1] - c * 0.75 * cos(th) : q[1] + c * 0.75 * cos(th),
                           q[2] - c * 0.75 * sin(th)};
            double cs = cos(psi), sn = sin(psi);
            double a[3] = {q[0] * cs - q[1] * sn, q[0] * sn + q[1] * cs, q[2]};
            double b[3] = {e[0] * cs - e[1] * sn, e[0] * sn + e[1] * cs, e[2]};
            /* fixed rotations about x, then y, then z, then the translation */
            double a1[3] = {a[0], a[1] * cos(thx) - a[2] * sin(thx), a[1] * sin(thx) + a[2] * cos(thx)};
            double b1[3] = {b[0], b[1] * cos(thx) - b[2] * sin(thx), b[1] * sin(thx) + b[2] * cos(thx)};
            double a2[3] = {a1[0] * cos(thy) + a1[2] * sin(thy), a1[1], -a1[0] * sin(thy) + a1[2] * cos(thy)};
            double b2[3] = {b1[0] * cos(thy) + b1[2] * sin(thy), b1[1], -b1[0] * sin(thy) + b1[2] * cos(thy)};
            double a3[3] = {a2[0] * cos(thz) - a2[1] * sin(thz), a2[0] * sin(thz) + a2[1] * cos(thz), a2[2]};
            double b3[3] = {b2[0] * cos(thz) - b2[1] * sin(thz), b2[0] * sin(thz) + b2[1] * cos(thz), b2[2]};
            for (int i = 0; i < 3; i++) {
                S->xyz[((size_t)k * nt + t) * 3 + i] = a3[i] + tr[i];
                S->xyzt[((size_t)k * nt + t) * 3 + i] = b3[i] + tr[i];
            }
        }
        for (int t = 0; t < nt; t++) {
            int tm = t == 0 ? nt - 1 : t - 1, tp = t == nt - 1 ? 0 : t + 1;
            const double* xp = S->xyz + ((size_t)k * nt + tp) * 3;
            const double* xm = S->xyz + ((size_t)k * nt + tm) * 3;
            const double* x0 = S->xyz + ((size_t)k * nt + t) * 3;
            const double* xt = S->xyzt + ((size_t)k * nt + t) * 3;
            double v[3], ch[3];
            for (int i = 0; i < 3; i++) v[i] = B->vinf[i] - (xp[i] - xm[i]) / (2 * B->dtau);
            for (int i = 0; i < 3; i++) ch[i] = xt[i] - x0[i];
            double l = sqrt(ch[0] * ch[0] + ch[1] * ch[1] + ch[2] * ch[2]);
            for (int i = 0; i < 3; i++) ch[i] = ch[i] / l;
            size_t p2 = (size_t)k * nt + t;
            double um = v[0] * ch[0] + v[1] * ch[1] + v[2] * ch[2];
            S->u[p2] = um;
            double mach = fabs(um / B->a0);
            double re = fabs(um * c / nu);
            int br[6];
            o_brackets(T, geo[4 * k], mach, re, br);
            for (int i = 0; i < T->na; i++) cl[i] = o_table_lookup(T, geo[4 * k], mach, re, br, 0, i);
            /* first AoA >= 0 deg, first AoA >= 6 deg, first cl > 0 (bb_core.cu:254-275);
             * an index that is never found stays 0, as in the zero-initialised build */
            int a1 = 0, a2 = 0, a3 = 0, f1 = 0, f2 = 0, f3 = 0;
            for (int i = 0; i < T->na; i++) {
                if (T->aoa[i] >= 0.0 && !f1) { a1 = i; f1 = 1; }
                if (T->aoa[i] >= 6.0 && !f2) { a2 = i; f2 = 1; }
                if (cl[i] > 0 && !f3) { a3 = i; f3 = 1; }
                if (f1 && f2 && f3) break;
            }
            double cla = (cl[a2] - cl[a1]) / (T->aoa[a2] - T->aoa[a1]);
            S->cla[p2] = cla;
            double w = (0 - T->aoa[a1 - 1]) / (T->aoa[a1] - T->aoa[a1 - 1]);
            double cl0 = cl[a1 - 1] * (1 - w) + cl[a1] * w;
            w = (0 - cl[a3 - 1]) / (cl[a3] - cl[a3 - 1]);
            double al0 = T->aoa[a3 - 1] * (1 - w) + T->aoa[a3] * w;
            /* fixed point for the effective angle (bb_core.cu:291-321) */
            double cn = bbd[((size_t)t * ns + k) * 7 + 4], ct = bbd[((size_t)t * ns + k) * 7 + 5];
            double ae = 0.0, err = 1;
            int it = 0;
            while (err > 1e-3) {
                double clsec = cn * cos(ae * M_PI / 180) - ct * sin(ae * M_PI / 180);
                double ae1 = (clsec - cl0) / cla;
                err = fabs(ae1 - ae);
                ae = ae1;
                it += 1;
                if (it > 50) break;
            }
            double al = fabs(ae - al0);
            S->alpha[p2] = al;
            double* bl = S->bl + p2 * 4;
            if (B->t_del == 0) {
                for (int i = 0; i < 4; i++) bl[i] = bbd[((size_t)t * ns + k) * 7 + i];
            } else if (B->t_del == 1) {
                /* table thicknesses at the bracketing AoA entries (bb_core.cu:357-413) */
                for (int i = 0; i < T->na; i++)
                    if (T->aoa[i] >= ae) { a1 = i; break; }
                double wa = (ae - T->aoa[a1 - 1]) / (T->aoa[a1] - T->aoa[a1 - 1]);
                double lo[4], hi[4];
                for (int i = 0; i < 4; i++) {
                    lo[i] = o_table_lookup(T, geo[4 * k], mach, re, br, i + 3, a1 - 1);
                    hi[i] = o_table_lookup(T, geo[4 * k], mach, re, br, i + 3, a1);
                }
                for (int i = 0; i < 4; i++) bl[i] = c * (lo[i] * (1 - wa) + hi[i] * wa);
            } else {
                /* empirical thicknesses (bb_core.cu:414-438) */
                double lr = log10(re);
                double d0 = c * pow(10.0, (1.6569 - 0.9045 * lr + 0.0596 * (lr * lr)));
                double ds0 = c * pow(10.0, (3.0187 - 1.5397 * lr + 0.1059 * (lr * lr)));
                bl[1] = d0 * pow(10.0, (-0.04175 * al + 0.00106 * (al * al)));
                bl[3] = ds0 * pow(10.0, (-0.0432 * al + 0.00113 * (al * al)));
                if (al <= 7.5) bl[0] = d0 * pow(10.0, (0.03114 * al));
                else if (al > 12.5) bl[0] = d0 * 12.0 * pow(10.0, 0.0258 * al);
                else bl[0] = d0 * 0.0303 * pow(10.0, 0.2336 * al);
                if (al <= 7.5) bl[2] = ds0 * pow(10.0, (0.0679 * al));
                else if (al > 12.5) bl[2] = ds0 * 52.42 * pow(10.0, 0.0258 * al);
                else bl[2] = ds0 * 0.0162 * pow(10.0, 0.3066 * al);
            }
        }
    }
    free(cl);
}

typedef struct {
    const acumo_bpm* B;
    o_bbsurf* S;
    int o0, o1, obs_base;
    const double* obs;
    double *spl, *oaspl;
} bpm_job;

/* Observer loop (bb_core.cu:449-557) and aggregation (bb_core.cu:563-583) for one shard;
 * output_tmp is kept per observer ([step][band][7]) since observers never mix. */
static void* o_bpm_shard(void* arg)
{
    bpm_job* J = (bpm_job*)arg;
    const acumo_bpm* B = J->B;
    int nt = B->ntime, nf = B->nf;
    double nu = 0.0000181206 / 1.22500;
    double* tmp = (double*)malloc(sizeof(double) * (size_t)nt * nf * 7);
    for (int io = J->o0; io < J->o1; io++) {
        const double* ob = J->obs + 3 * io;
        for (size_t i = 0; i < (size_t)nt * nf * 7; i++) tmp[i] = -100.0;
        int xs = 0;
        for (int is = 0; is < B->nsurf; is++) {
            int ns = B->nsect[is];
            const double* geo = B->xyzcR + 4 * (size_t)xs;
            const o_bbsurf* S = J->S + is;
            double span = B->span[is];
            for (int k = 0; k < ns; k++) {
                double ls;
                if (k == 0) ls = (geo[4 * (k + 1)] - geo[4 * k]) / 2.0 * span;
                else if (k == ns - 1) ls = (geo[4 * k] - geo[4 * (k - 1)]) / 2.0 * span;
                else ls = (geo[4 * (k + 1)] - geo[4 * (k - 1)]) / 2.0 * span;
                double c = geo[4 * k + 3] * span;
                int km = k == ns - 1 ? k - 1 : k, kp = k == ns - 1 ? k : k + 1;
                for (int t = 0; t < nt; t++) {
                    size_t p2 = (size_t)k * nt + t;
                    const double* x0 = S->xyz + p2 * 3;
                    const double* xt = S->xyzt + p2 * 3;
                    double tr[3][3], n;
                    /* chordwise, spanwise and normal unit vectors (bb_core.cu:473-513) */
                    for (int i = 0; i < 3; i++) tr[0][i] = xt[i] - x0[i];
                    n = sqrt(tr[0][0] * tr[0][0] + tr[0][1] * tr[0][1] + tr[0][2] * tr[0][2]);
                    for (int i = 0; i < 3; i++) tr[0][i] = tr[0][i] / n;
                    for (int i = 0; i < 3; i++)
                        tr[1][i] = S->xyz[((size_t)kp * nt + t) * 3 + i] - S->xyz[((size_t)km * nt + t) * 3 + i];
                    n = sqrt(tr[1][0] * tr[1][0] + tr[1][1] * tr[1][1] + tr[1][2] * tr[1][2]);
                    for (int i = 0; i < 3; i++) tr[1][i] = tr[1][i] / n;
                    if (B->ccw[is] == 1) {
                        tr[2][0] = tr[0][1] * tr[1][2] - tr[0][2] * tr[1][1];
                        tr[2][1] = tr[0][2] * tr[1][0] - tr[0][0] * tr[1][2];
                        tr[2][2] = tr[0][0] * tr[1][1] - tr[0][1] * tr[1][0];
                        n = sqrt(tr[2][0] * tr[2][0] + tr[2][1] * tr[2][1] + tr[2][2] * tr[2][2]);
                        for (int i = 0; i < 3; i++) tr[2][i] = tr[2][i] / n;
                    } else {
                        tr[2][0] = tr[1][1] * tr[0][2] - tr[1][2] * tr[0][1];
                        tr[2][1] = tr[1][2] * tr[0][0] - tr[1][0] * tr[0][2];
                        tr[2][2] = tr[1][0] * tr[0][1] - tr[1][1] * tr[0][0];
                        n = sqrt(tr[2][0] * tr[2][0] + tr[2][1] * tr[2][1] + tr[2][2] * tr[2][2]);
                        /* the clockwise branch divides by the square root of the norm
                         * (bb_core.cu:510-512); kept as the reference has it */
                        for (int i = 0; i < 3; i++) tr[2][i] = tr[2][i] / sqrt(n);
                    }
                    /* convected emission time and source-observer geometry
                     * (bb_core.cu:515-530); aa_mode 1 reproduces aa = 0 */
                    double rp[3];
                    for (int i = 0; i < 3; i++) rp[i] = ob[i] - xt[i];
                    double aMv = B->a0 * B->a0 - B->vinf[0] * B->vinf[0] - B->vinf[1] * B->vinf[1] -
                                 B->vinf[2] * B->vinf[2];
                    double bb = rp[0] * B->vinf[0] + rp[1] * B->vinf[1] + rp[2] * B->vinf[2];
                    double cc = rp[0] * rp[0] + rp[1] * rp[1] + rp[2] * rp[2];
                    double aa = B->aa_mode == 1 ? 0.0 : aMv;
                    double tau = (-bb + sqrt(bb * bb + aa * cc)) / aMv;
                    for (int i = 0; i < 3; i++) rp[i] = ob[i] - xt[i] - B->vinf[i] * tau;
                    double rpn = sqrt(rp[0] * rp[0] + rp[1] * rp[1] + rp[2] * rp[2]);
                    double r2[3];
                    for (int i = 0; i < 3; i++) r2[i] = rp[0] * tr[i][0] + rp[1] * tr[i][1] + rp[2] * tr[i][2];
                    double re_ = sqrt(r2[1] * r2[1] + r2[2] * r2[2]);
                    double th = acos(fabs(r2[0] / rpn));
                    double ph = acos(fabs(r2[1]) / re_);
                    const double* bl = S->bl + p2 * 4;
                    acumo_bpm_core(rpn, th, ph, c, ls, fabs(S->alpha[p2]), S->u[p2], nu, B->a0, B->trip[is], bl[0],
                                   bl[1], bl[2], bl[3], k, ns, B->ff, nf, span, tmp + (size_t)t * nf * 7);
                }
            }
            xs += ns;
        }
        /* energy mean over steps and band sum (bb_core.cu:563-583) */
        int oo = io - J->obs_base;
        double* sp = J->spl + (size_t)oo * nf * 7;
        for (int f = 0; f < nf; f++) {
            for (int c = 0; c < 7; c++) {
                double v = sp[f * 7 + c];
                for (int t = 0; t < nt; t++) v = db_add(v, tmp[((size_t)t * nf + f) * 7 + c]);
                sp[f * 7 + c] = 10.0 * log10(pow(10.0, (v / 10.0)) / (double)nt);
            }
            J->oaspl[oo] = db_add(J->oaspl[oo], sp[f * 7]);
        }
    }
    free(tmp);
    return NULL;
}

/* findBBnoise (bb_core.cu:11-586) over observers [obs0, obs0+nob).  spl[nob][nf][7] and
 * oaspl[nob] must arrive seeded (-100 dB in the reference driver, main.cu:132-142). */
int acumo_bpm_run(const acumo_bpm* B, const double* obs, int obs0, int nob, double* spl, double* oaspl, int nthreads)
{
    int nt = B->ntime;
    o_bbsurf* S = (o_bbsurf*)calloc((size_t)B->nsurf, sizeof(o_bbsurf));
    int xs = 0, as = 0, ss = 0, ms = 0, rs = 0;
    size_t ds = 0, dt = 0;
    for (int is = 0; is < B->nsurf; is++) {
        int ns = B->nsect[is];
        size_t n = (size_t)ns * nt;
        S[is].xyz = (double*)malloc(sizeof(double) * n * 3);
        S[is].xyzt = (double*)malloc(sizeof(double) * n * 3);
        S[is].u = (double*)malloc(sizeof(double) * n);
        S[is].alpha = (double*)malloc(sizeof(double) * n);
        S[is].cla = (double*)malloc(sizeof(double) * n);
        S[is].bl = (double*)malloc(sizeof(double) * n * 4);
        o_table T;
        T.ns = B->nsect_t[is]; T.na = B->naoa_t[is]; T.nm = B->nmach_t[is]; T.nr = B->nre_t[is];
        T.sect = B->sect_t + ss; T.aoa = B->aoa_t + as; T.mach = B->mach_t + ms; T.re = B->re_t + rs;
        T.data = B->bbdata_t + dt;
        o_bpm_surface_prep(B, is, B->xyzcR + 4 * (size_t)xs, B->bbdata + ds, &T, &S[is]);
        xs += ns;
        ds += (size_t)ns * nt * 7;
        ss += T.ns; as += T.na; ms += T.nm; rs += T.nr;
        dt += (size_t)T.ns * T.na * T.nm * T.nr * 7;
    }
    if (nthreads < 1) nthreads = 1;
    if (nthreads > nob) nthreads = nob;
    bpm_job* jobs = (bpm_job*)calloc((size_t)nthreads, sizeof(bpm_job));
    pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
    for (int k = 0; k < nthreads; k++) {
        jobs[k].B = B;
        jobs[k].S = S;
        jobs[k].obs = obs;
        jobs[k].o0 = obs0 + (int)((long)nob * k / nthreads);
        jobs[k].o1 = obs0 + (int)((long)nob * (k + 1) / nthreads);
        jobs[k].obs_base = obs0;
        jobs[k].spl = spl;
        jobs[k].oaspl = oaspl;
    }
    for (int k = 1; k < nthreads; k++) pthread_create(&th[k], NULL, o_bpm_shard, &jobs[k]);
    o_bpm_shard(&jobs[0]);
    for (int k = 1; k < nthreads; k++) pthread_join(th[k], NULL);
    for (int is = 0; is < B->nsurf; is++) {
        free(S[is].xyz); free(S[is].xyzt); free(S[is].u); free(S[is].alpha); free(S[is].cla); free(S[is].bl);
    }
    free(S);
    free(jobs);
    free(th);
    return 0;
}

/* Exposes the per-(section, step) state for pinning: u, alpha, cl_alpha [sect][step] and
 * bl [sect][step][4] of BB surface `is`. */
int acumo_bpm_prep(const acumo_bpm* B, int is_req, double* u, double* alpha, double* cla, double* bl)
{
    int xs = 0, as = 0, ss = 0, ms = 0, rs = 0;
    size_t ds = 0, dt = 0;
    for (int is = 0; is < B->nsurf; is++) {
        int ns = B->nsect[is];
        o_table T;
        T.ns = B->nsect_t[is]; T.na = B->naoa_t[is]; T.nm = B->nmach_t[is]; T.nr = B->nre_t[is];
        T.sect = B->sect_t + ss; T.aoa = B->aoa_t + as; T.mach = B->mach_t + ms; T.re = B->re_t + rs;
        T.data = B->bbdata_t + dt;
        if (is == is_req) {
            size_t n = (size_t)ns * B->ntime;
            o_bbsurf S;
            S.xyz = (double*)malloc(sizeof(double) * n * 3);
            S.xyzt = (double*)malloc(sizeof(double) * n * 3);
            S.u = u; S.alpha = alpha; S.cla = cla; S.bl = bl;
            o_bpm_surface_prep(B, is, B->xyzcR + 4 * (size_t)xs, B->bbdata + ds, &T, &S);
            free(S.xyz); free(S.xyzt);
            return 0;
        }
        xs += ns;
        ds += (size_t)ns * B->ntime * 7;
        ss += T.ns; as += T.na; ms += T.nm; rs += T.nr;
        dt += (size_t)T.ns * T.na * T.nm * T.nr * 7;
    }
    return -1;
}

/* Exposes the blade positions of BB surface `is`: quarter chord xyz and trailing edge
 * xyzt, each [sect][step][3] (bb_core.cu:79-164). */
int acumo_bpm_geom(const acumo_bpm* B, int is_req, double* xyz, double* xyzt)
{
    int xs = 0, as = 0, ss = 0, ms = 0, rs = 0;
    size_t ds = 0, dt = 0;
    for (int is = 0; is < B->nsurf; is++) {
        int ns = B->nsect[is];
        o_table T;
        T.ns = B->nsect_t[is]; T.na = B->naoa_t[is]; T.nm = B->nmach_t[is]; T.nr = B->nre_t[is];
        T.sect = B->sect_t + ss; T.aoa = B->aoa_t + as; T.mach = B->mach_t + ms; T.re = B->re_t + rs;
        T.data = B->bbdata_t + dt;
        if (is == is_req) {
            size_t n = (size_t)ns * B->ntime;
            o_bbsurf S;
            S.xyz = xyz; S.xyzt = xyzt;
            S.u = (double*)malloc(sizeof(double) * n); S.alpha = (double*)malloc(sizeof(double) * n);
            S.cla = (double*)malloc(sizeof(double) * n); S.bl = (double*)malloc(sizeof(double) * n * 4);
            o_bpm_surface_prep(B, is, B->xyzcR + 4 * (size_t)xs, B->bbdata + ds, &T, &S);
            free(S.u); free(S.alpha); free(S.cla); free(S.bl);
            return 0;
        }
        xs += ns;
        ds += (size_t)ns * B->ntime * 7;
        ss += T.ns; as += T.na; ms += T.nm; rs += T.nr;
        dt += (size_t)T.ns * T.na * T.nm * T.nr * 7;
    }
    return -1;
}
