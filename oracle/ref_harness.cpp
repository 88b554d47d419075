/*
 * ref_harness.cpp -- extern "C" entry points around the reference's own sources compiled
 * as host C++ by oracle/build_ref.sh (see ref_shim.h for how the sources are compiled).
 *
 * TEST INFRASTRUCTURE ONLY: the oracle tests load oracle/_ref/libacumref_{f32,f64}.so to
 * pin the C restatement in oracle/acum_oracle.c and to generate the golden fixtures
 * under tests/golden/.  The product never links or loads this file.
 *
 * The harness replays what main.cu does around the two hot-path calls, minus CUDA:
 *   read_inputs / read_BB_inputs / read_observers / read_surf     (main.cu:56-78)
 *   preprocess_imper                                             (main.cu:88)
 *   tObs[t] = t*dPsi, pT/pL/pA zeroed, BBspl/BBoaspl set to -100   (main.cu:122-142)
 *   findBBnoise(...)                                             (main.cu:150)
 *   findPressureTimeHistory(...) run serially on the host        (main.cu:236)
 * Every array crosses this boundary as double; in the FP32 build values are narrowed to
 * float on the way in (all fixtures hold float32-exact values, so nothing is lost).
 */
#include <unistd.h>
#include <fcntl.h>

#include "variables.cuh"
#include "io.cuh"
#include "preprocess.cuh"
#include "core.cuh"
#include "bb_core.cuh"
#include "bb_utils.cuh"
#include "mathfunc.cuh"

typedef float real; /* `float` is `double` in the FP64 build (ref_shim.h) */

void* acum_ref_malloc(size_t n) { return (malloc)(n < 4096 ? 4096 : n); }

#ifdef ACUM_REF_F64
#undef fscanf
int acum_ref_fscanf(FILE* f, const char* fmt, ...)
{
    char buf[1024];
    size_t j = 0;
    for (size_t i = 0; fmt[i] && j + 3 < sizeof(buf);) {
        char c = fmt[i++];
        buf[j++] = c;
        if (c != '%') continue;
        if (fmt[i] == '%') { buf[j++] = fmt[i++]; continue; }
        int suppressed = 0;
        while (fmt[i] == '*' || (fmt[i] >= '0' && fmt[i] <= '9')) {
            if (fmt[i] == '*') suppressed = 1;
            buf[j++] = fmt[i++];
        }
        char k = fmt[i];
        if (!suppressed && (k == 'f' || k == 'e' || k == 'g' || k == 'E' || k == 'G')) buf[j++] = 'l';
    }
    buf[j] = 0;
    va_list ap;
    va_start(ap, fmt);
    int r = vfscanf(f, buf, ap);
    va_end(ap);
    return r;
}
#endif

static int g_saved_fd = -1;
static void quiet_on(int q)
{
    if (!q) return;
    fflush(stdout);
    g_saved_fd = dup(1);
    int fd = open("/dev/null", O_WRONLY);
    if (fd >= 0) { dup2(fd, 1); close(fd); }
}
static void quiet_off(int q)
{
    if (!q || g_saved_fd < 0) return;
    fflush(stdout);
    dup2(g_saved_fd, 1);
    close(g_saved_fd);
    g_saved_fd = -1;
}

extern "C" int acumref_real_bytes(void) { return (int)sizeof(real); }

/* Reads a deck directory with the reference's own readers (main.cu:56-78). */
extern "C" int acumref_load(const char* dir, int quiet)
{
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) return -1;
    if (chdir(dir) != 0) return -2;
    quiet_on(quiet);
    read_inputs("input");
    if (BB_noise == 1) read_BB_inputs("input_BB");
    read_observers("obs.dat");
    read_surf(nSurf);
    quiet_off(quiet);
    if (chdir(cwd) != 0) return -3;
    return 0;
}

extern "C" void acumref_dims(int* d)
{
    int et = 0;
    for (int i = 0; i < nSurf; i++) et += E[i];
    d[0] = nSurf; d[1] = nTime; d[2] = nObs; d[3] = et;
    d[4] = BB_noise; d[5] = nSurf_BB; d[6] = nf2; d[7] = t_del;
    d[8] = impermeable; d[9] = periodic; d[10] = lowpass; d[11] = nPRham;
}

extern "C" void acumref_surf_sizes(int* e)
{
    for (int i = 0; i < nSurf; i++) e[i] = E[i];
}

extern "C" void acumref_scalars(double* s)
{
    s[0] = a0; s[1] = rhoRef; s[2] = pRef; s[3] = oM; s[4] = dPsi; s[5] = dTau;
    s[6] = vInf[0]; s[7] = vInf[1]; s[8] = vInf[2]; s[9] = Minf; s[10] = Mref;
    s[11] = CFDscale; s[12] = OBSscale; s[13] = xy_angle; s[14] = xz_angle;
}

extern "C" void acumref_observers(double* r)
{
    for (int i = 0; i < 3 * nObs; i++) r[i] = rObs[i];
}

extern "C" void acumref_field_sizes(long* s)
{
    s[0] = nXtot; s[1] = nNtot; s[2] = nVtot; s[3] = nPRtot;
}

/* The AoS arrays of variables.cu:54 (after read_surf, and after preprocess_imper). */
extern "C" void acumref_fields(double* X, double* N, double* V, double* PR)
{
    for (long i = 0; i < nXtot; i++) X[i] = Xham[i];
    for (long i = 0; i < nNtot; i++) N[i] = Nham[i];
    for (long i = 0; i < nVtot; i++) V[i] = Vham[i];
    for (long i = 0; i < nPRtot; i++) PR[i] = PRham[i];
}

extern "C" int acumref_preprocess(int quiet)
{
    if (impermeable != 1) return -1;
    quiet_on(quiet);
    preprocess_imper();
    quiet_off(quiet);
    return 0;
}

/* Serial run of findPressureTimeHistory (core.cu:18) over observers
 * [obs0, obs0+nob); outputs are [nTime][nob] (main.cu:123-130 layout). */
extern "C" int acumref_tonal(int obs0, int nob, double* pTo, double* pLo, double* pAo, int quiet)
{
    if (obs0 < 0 || nob <= 0 || obs0 + nob > nObs) return -1;
    size_t n = (size_t)nTime * nob;
    real* pT = (real*)calloc(n, sizeof(real));
    real* pL = (real*)calloc(n, sizeof(real));
    real* pA = (real*)calloc(n, sizeof(real));
    real* tO = (real*)calloc(nTime, sizeof(real));
    for (int t = 0; t < nTime; t++) tO[t] = t * dPsi;
    quiet_on(quiet);
    findPressureTimeHistory(rObs + 3 * obs0, tO, pT, pL, pA, Xham, Nham, Vham, PRham, nSurf, XPtr, NPtr,
                            VPtr, PRPtr, E, nob, nTime, dPsi, dTau, a0, rhoRef, vInf, oM);
    quiet_off(quiet);
    for (size_t i = 0; i < n; i++) { pTo[i] = pT[i]; pLo[i] = pL[i]; pAo[i] = pA[i]; }
    free(pT); free(pL); free(pA); free(tO);
    return 0;
}

/* findBBnoise (bb_core.cu:11) over observers [obs0, obs0+nob); outputs are
 * BBspl[nob][nf2][7] and BBoaspl[nob], both seeded with -100 dB as main.cu:132-142. */
extern "C" int acumref_bpm(int obs0, int nob, double* splo, double* oaslo, int quiet)
{
    if (BB_noise != 1 || obs0 < 0 || nob <= 0 || obs0 + nob > nObs) return -1;
    size_t ns = (size_t)nob * nf2 * 7;
    real* spl = (real*)calloc(ns, sizeof(real));
    real* oas = (real*)calloc(nob, sizeof(real));
    real* tO = (real*)calloc(nTime, sizeof(real));
    for (int t = 0; t < nTime; t++) tO[t] = t * dPsi;
    for (size_t i = 0; i < ns; i++) spl[i] = -100.0;
    for (int i = 0; i < nob; i++) oas[i] = -100.0;
    quiet_on(quiet);
    findBBnoise(nSurf_BB, nob, nTime, dTau, span, omega, ccw, psi_offset, trip, rotate, translate, xsPtr, dsPtr,
                nsect, xyzcR, bbdata, nsect_t, nmach_t, naoa_t, nre_t, aPtr, mPtr, rPtr, sPtr, dPtr, sect_t, mach_t,
                aoa_t, re_t, bbdata_t, t_del, vInf, rObs + 3 * obs0, tO, nf2, ff, a0, spl, oas);
    quiet_off(quiet);
    for (size_t i = 0; i < ns; i++) splo[i] = spl[i];
    for (int i = 0; i < nob; i++) oaslo[i] = oas[i];
    free(spl); free(oas); free(tO);
    return 0;
}

/* ---- single functions, for golden vectors ---- */

extern "C" void acumref_bb_curve(int which, const double* x, double* y, int n)
{
    real* a = (real*)calloc(n, sizeof(real));
    real* b = (real*)calloc(n, sizeof(real));
    for (int i = 0; i < n; i++) a[i] = x[i];
    if (which == 0) a_min(a, b, n);
    else if (which == 1) a_max(a, b, n);
    else if (which == 2) b_min(a, b, n);
    else b_max(a, b, n);
    for (int i = 0; i < n; i++) y[i] = b[i];
    free(a); free(b);
}

extern "C" double acumref_g5comp(double h, double eta) { return g5comp(h, eta); }

extern "C" void acumref_make_periodic(double* f, int n)
{
    real* g = (real*)calloc(n, sizeof(real));
    real* fc = (real*)calloc(n + 1, sizeof(real));
    for (int i = 0; i < n; i++) g[i] = f[i];
    make_periodic(g, n, 0, fc);
    for (int i = 0; i < n; i++) f[i] = g[i];
    free(g); free(fc);
}

extern "C" void acumref_lowpass(double* f, int n)
{
    /* preprocess.cu:285 and 323-333: two passes of (3-point median, 13-tap Gaussian) */
    real* g = (real*)calloc(n, sizeof(real));
    real gauss[13];
    for (int i = 0; i < n; i++) g[i] = f[i];
    pre_gaussfilt1(gauss, 13);
    for (int k = 0; k < 2; k++) {
        medfilt1(g, n);
        gaussfilt1(g, gauss, n, 13);
    }
    for (int i = 0; i < n; i++) f[i] = g[i];
    free(g);
}

extern "C" void acumref_differentiate(const double* u, double* ud, double dt, int n, int biased)
{
    real* a = (real*)calloc(n, sizeof(real));
    real* b = (real*)calloc(n, sizeof(real));
    for (int i = 0; i < n; i++) a[i] = u[i];
    if (biased) differentiate_biased(a, b, dt, n);
    else differentiate(a, b, dt, n);
    for (int i = 0; i < n; i++) ud[i] = b[i];
    free(a); free(b);
}

/* core() of bb_core.cu:591 for one (observer, section, step); needs a loaded BB deck for
 * the band table ff.  out[nf2*7] starts at -100 dB like output_tmp (bb_core.cu:40). */
extern "C" int acumref_core(const double* s, int trip_, int isect, int nsect_, double* out)
{
    if (BB_noise != 1) return -1;
    real* o = (real*)calloc((size_t)nf2 * 7, sizeof(real));
    for (int i = 0; i < nf2 * 7; i++) o[i] = -100.0;
    /* s = rpnorm, theta, phi, c, lsect, alpha, u, nu, a0, del_s, del_p, dis_s, dis_p, cl_alpha, R */
    core(s[0], s[1], s[2], s[3], s[4], s[5], s[6], s[7], s[8], trip_, s[9], s[10], s[11], s[12], isect, 0, 0, o, 1,
         nf2, nsect_, 0, ff, s[13], s[14]);
    for (int i = 0; i < nf2 * 7; i++) out[i] = o[i];
    free(o);
    return 0;
}

extern "C" void acumref_bands(double* f)
{
    for (int i = 0; i < nf2; i++) f[i] = ff[i];
}

/* preprocess_per (preprocess.cu:8-226), the permeable surfaces' preprocessing, on caller
 * arrays laid out as [element][step][k] per surface, surface after surface (X k = 4, N 6,
 * V 6, U 6, PR 4 = P, dP, rho, drho): the reference's globals are set as its reader and
 * main.cu:87 leave them (impermeable = 0, nPRham = 4), the function runs, the arrays
 * come back.  scal = dTau, a0, rhoRef, Mref, CFDscale. */
extern "C" int acumref_preprocess_per(int nsurf, const int* ne, int nt, const double* scal, int periodic_,
                                      int lowpass_, double* X, double* N, double* V, double* U, double* PR,
                                      int quiet)
{
    if (nsurf <= 0 || nt < 4) return -1;
    long etot_ = 0;
    for (int i = 0; i < nsurf; i++) etot_ += ne[i];
    nSurf = nsurf;
    nTime = nt;
    dTau = scal[0];
    a0 = scal[1];
    rhoRef = scal[2];
    Mref = scal[3];
    CFDscale = scal[4];
    periodic = periodic_;
    lowpass = lowpass_;
    impermeable = 0;
    nPRham = 4;
    E = (int*)calloc(nsurf, sizeof(int));
    XPtr = (int*)calloc(nsurf, sizeof(int));
    NPtr = (int*)calloc(nsurf, sizeof(int));
    VPtr = (int*)calloc(nsurf, sizeof(int));
    UPtr = (int*)calloc(nsurf, sizeof(int));
    PRPtr = (int*)calloc(nsurf, sizeof(int));
    long off = 0;
    for (int i = 0; i < nsurf; i++) {
        E[i] = ne[i];
        XPtr[i] = (int)(off * nt * 4);
        NPtr[i] = (int)(off * nt * 6);
        VPtr[i] = (int)(off * nt * 6);
        UPtr[i] = (int)(off * nt * 6);
        PRPtr[i] = (int)(off * nt * 4);
        off += ne[i];
    }
    const long n = etot_ * nt;
    Xham = (real*)calloc(n * 4, sizeof(real));
    Nham = (real*)calloc(n * 6, sizeof(real));
    Vham = (real*)calloc(n * 6, sizeof(real));
    Uham = (real*)calloc(n * 6, sizeof(real));
    PRham = (real*)calloc(n * 4, sizeof(real));
    for (long i = 0; i < n * 4; i++) Xham[i] = X[i];
    for (long i = 0; i < n * 6; i++) { Nham[i] = N[i]; Vham[i] = V[i]; Uham[i] = U[i]; }
    for (long i = 0; i < n * 4; i++) PRham[i] = PR[i];
    quiet_on(quiet);
    preprocess_per();
    quiet_off(quiet);
    for (long i = 0; i < n * 4; i++) X[i] = Xham[i];
    for (long i = 0; i < n * 6; i++) { N[i] = Nham[i]; V[i] = Vham[i]; U[i] = Uham[i]; }
    for (long i = 0; i < n * 4; i++) PR[i] = PRham[i];
    free(Xham); free(Nham); free(Vham); free(Uham); free(PRham);
    free(E); free(XPtr); free(NPtr); free(VPtr); free(UPtr); free(PRPtr);
    Xham = Nham = Vham = Uham = PRham = NULL;
    E = XPtr = NPtr = VPtr = UPtr = PRPtr = NULL;
    return 0;
}

/* preprocess_per (main.cu:87) on the deck loaded by acumref_load (a permeable deck:
 * read_surf filled Xham, Uham, PRham and Nham from the 12-column rows, io.cu:263-293). */
extern "C" int acumref_preprocess_per_loaded(int quiet)
{
    if (impermeable != 0) return -1;
    quiet_on(quiet);
    preprocess_per();
    quiet_off(quiet);
    return 0;
}

/* The five AoS arrays of a loaded permeable deck (Xham, Nham, Vham, Uham, PRham; sizes
 * nXtot, nNtot, nVtot, nUtot, nPRtot with nPRham = 4). */
extern "C" void acumref_fields_per(double* X, double* N, double* V, double* U, double* PR)
{
    for (long i = 0; i < nXtot; i++) X[i] = Xham[i];
    for (long i = 0; i < nNtot; i++) N[i] = Nham[i];
    for (long i = 0; i < nVtot; i++) V[i] = Vham[i];
    for (long i = 0; i < nUtot; i++) U[i] = Uham[i];
    for (long i = 0; i < nPRtot; i++) PR[i] = PRham[i];
}

/* The reference's writer (io.cu:137-203) run in `dir` on the zeroed pT/pL/pA that
 * main.cu:123-130 prepares, which is what it writes for a permeable deck (main.cu:236
 * launches no kernel for it). */
extern "C" int acumref_write_zero_history(const char* dir)
{
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) return -1;
    if (chdir(dir) != 0) return -2;
    real* z = (real*)calloc((size_t)nTime * nObs, sizeof(real));
    writeTimeHistory(z, z, z);
    free(z);
    if (chdir(cwd) != 0) return -3;
    return 0;
}
