// bpm.cu -- sm_103a kernels of the broadband (BPM) path and its C ABI entry points.
//
// The reference evaluates, for every observer x span section x source step, the BPM
// sub-models over 42 bands and log-adds the seven component levels in dB
// (bb_core.cu:449-583, core() at 591-1043).  Every component level has the form
//     L = 10 log10(D * A) (+ clip)   with  D = d(theta, phi) / r^2
// where only the directivity-over-distance factor D depends on the observer and the
// amplitude A depends on (section, step, band) alone.  The GPU path therefore splits the
// work three ways:
//
//  bb_pos_kernel / bb_prep_kernel   per (section, step), FP64: blade kinematics, chordwise
//      flow speed, table lookups, the fixed-point effective angle of attack and the
//      boundary-layer thicknesses (bb_core.cu:60-444), the chord/span/normal frame, and
//      every band-independent scalar of core() -- the branch decisions of the model are
//      taken here in FP64.
//  bb_spec_kernel    per (section, step, band), FP32: the spectral amplitudes A of the six
//      sub-model components (TBL-TE suction/pressure/separation, LBL-VS, TEB-VS, tip).
//  bb_obs_kernel     per (observer, section, step, band): D from the observer geometry
//      (once per (observer, section, step), shared by all bands through shared memory),
//      then the energies max(D*A, 1e-10) (the reference's -100 dB clip) summed over
//      sections and steps in FP32 partial sums folded into FP64; lane = observer and
//      warp = band pair, so each amplitude is read once per warp as a shared-memory
//      broadcast and one packed FP32 instruction covers both bands.
//  bb_final_kernel   the energy means over steps per (observer, band), in FP64 dB
//  bb_oaspl_kernel   the band sum (OASPL) per observer
//      (bb_core.cu:563-583).
//
// The reference's repeated dB log-adds become plain energy sums, which removes most of
// its transcendental work; the results are equal up to rounding.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "acum_internal.h"
#include "ctx.h"
#include "ptx.h"

namespace acum {

constexpr int kMaxAoa = 64;
constexpr int kSc = 32;    // spectral scalars per (section, step)
constexpr int kGeo = 16;   // geometry record per (section, step)
constexpr int kAmp = 8;    // amplitudes per (section, step, band)

struct BBSurfDev {
    double span, omega, psi_off, rot[3], tr[3];
    int ccw, trip, nsect, sec0;
    long long data_off;
    int ns_t, na_t, nm_t, nr_t;
    int sect_off, aoa_off, mach_off, re_off;
    long long tab_off;
};

struct BpmState {
    int S = 0, nbb = 0, O = 0, T = 0;
    DBuf<BBSurfDev> surf;
    DBuf<int> secsurf, secloc;
    DBuf<double> geom, data, sect_t, aoa_t, mach_t, re_t, table, pos, spl, oaspl, seed_spl, seed_oas, ff;
    DBuf<double> sums;
    DBuf<float> geo, sc, amp;
    bool uploaded = false;
};

static BpmState* state(acum_ctx* c)
{
    if (!c->bpm_state) c->bpm_state = new BpmState();
    return reinterpret_cast<BpmState*>(c->bpm_state);
}

void release_bpm_state(acum_ctx* c)
{
    if (!c->bpm_state) return;
    BpmState* s = state(c);
    s->surf.release(); s->secsurf.release(); s->secloc.release();
    s->geom.release(); s->data.release(); s->sect_t.release(); s->aoa_t.release(); s->mach_t.release();
    s->re_t.release(); s->table.release(); s->pos.release(); s->spl.release(); s->oaspl.release();
    s->seed_spl.release(); s->seed_oas.release(); s->ff.release(); s->sums.release();
    s->geo.release(); s->sc.release(); s->amp.release();
    delete s;
    c->bpm_state = nullptr;
}

// ----------------------------------------------------------- model pieces (FP64)

// bb_utils.cu:6-88 -- spectral shape curves A_min, A_max, B_min, B_max
template <typename R>
__device__ __forceinline__ R amin_(R a)
{
    if (a < (R)0.204) return sqrt((R)67.552 - (R)886.788 * (a * a)) - (R)8.219;
    if (a > (R)0.244) return (R)-142.795 * (a * a * a) + (R)103.656 * (a * a) - (R)57.757 * a + (R)6.006;
    return (R)-32.665 * a + (R)3.981;
}
template <typename R>
__device__ __forceinline__ R amax_(R a)
{
    if (a < (R)0.13) return sqrt((R)67.552 - (R)886.788 * (a * a)) - (R)8.219;
    if (a > (R)0.321) return (R)-4.669 * (a * a * a) + (R)3.491 * (a * a) - (R)16.699 * a + (R)1.149;
    return (R)-15.901 * a + (R)1.098;
}
template <typename R>
__device__ __forceinline__ R bmin_(R b)
{
    if (b < (R)0.13) return sqrt((R)16.888 - (R)886.788 * (b * b)) - (R)4.109;
    if (b > (R)0.145) return (R)-817.810 * (b * b * b) + (R)355.21 * (b * b) - (R)135.024 * b + (R)10.619;
    return (R)-83.607 * b + (R)8.138;
}
template <typename R>
__device__ __forceinline__ R bmax_(R b)
{
    if (b < (R)0.1) return sqrt((R)16.888 - (R)886.788 * (b * b)) - (R)4.109;
    if (b > (R)0.187) return (R)-80.541 * (b * b * b) + (R)44.174 * (b * b) - (R)39.381 * b + (R)2.344;
    return (R)-31.313 * b + (R)1.854;
}
// bb_utils.cu:90-121 -- bluntness shape G5
template <typename R>
__device__ __forceinline__ R g5_(R h, R eta)
{
    R mu, m;
    if (h <= (R)0.25) mu = (R)0.1211;
    else if (h <= (R)0.62) mu = (R)-0.2175 * h + (R)0.1755;
    else if (h < (R)1.15) mu = (R)-0.0308 * h + (R)0.0596;
    else mu = (R)0.0242;
    if (h <= (R)0.02) m = 0;
    else if (h < (R)0.5) m = (R)68.724 * h - (R)1.35;
    else if (h <= (R)0.62) m = (R)308.475 * h - (R)121.23;
    else if (h <= (R)1.15) m = (R)224.811 * h - (R)69.354;
    else if (h < (R)1.2) m = (R)1583.28 * h - (R)1631.592;
    else m = (R)268.344;
    if (m < 0) m = 0;
    const R eta0 = -sqrt((m * m * (mu * mu * mu * mu)) / ((R)6.25 + m * m * mu * mu));
    const R k = (R)2.5 * sqrt((R)1.0 - (eta0 / mu) * (eta0 / mu)) - (R)2.5 - m * eta0;
    if (eta <= eta0) return m * eta + k;
    if (eta <= 0) return (R)2.5 * sqrt((R)1.0 - (eta / mu) * (eta / mu)) - (R)2.5;
    if (eta <= (R)0.03616) return sqrt((R)1.5625 - (R)1194.99 * (eta * eta)) - (R)1.25;
    return (R)-155.543 * eta + (R)4.375;
}

__device__ __forceinline__ int count_le(const double* a, int n, double x)
{
    int k = 0;
    while (k < n && !(x < a[k])) ++k;
    return k;
}

struct BBDev {
    const BBSurfDev* surf;
    const int *secsurf, *secloc;
    const double *geom, *data, *sect_t, *aoa_t, *mach_t, *re_t, *table;
    double* pos;  // [S][T][6] quarter chord xyz, trailing edge xyz
    float* geo;   // [S*T][16]
    float* sc;    // [S*T][32]
    int S, T;
    double dtau, a0, vinf[3];
    int t_del;
};

// quarter-chord and trailing-edge positions (bb_core.cu:79-164)
__global__ void bb_pos_kernel(BBDev d)
{
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)d.S * d.T) return;
    const int gs = (int)(id / d.T), t = (int)(id % d.T);
    const BBSurfDev& su = d.surf[d.secsurf[gs]];
    const int k = d.secloc[gs], ns = su.nsect;
    const double* geo = d.geom + 4 * (size_t)su.sec0;
    const double span = su.span;
    // the y, z of section round(0.75 nsect) (bb_core.cu:88); nsect >= 3 keeps it in range
    const int i75 = min((int)round(ns * 0.75), ns - 1);
    const double c = geo[4 * k + 3] * span;
    double q[3] = {geo[4 * k] * span, geo[4 * i75 + 1] * span, geo[4 * i75 + 2] * span};
    if (su.ccw == 0) q[1] = -q[1];
    double psi = (d.dtau * t * su.omega + su.psi_off * M_PI / 180);
    if (su.ccw == 0) psi = -psi;
    const double th = d.data[su.data_off + ((size_t)t * ns + k) * 7 + 6] * M_PI / 180;
    const double e[3] = {q[0], su.ccw == 1 ? q[1] - c * 0.75 * cos(th) : q[1] + c * 0.75 * cos(th),
                         q[2] - c * 0.75 * sin(th)};
    const double cs = cos(psi), sn = sin(psi);
    const double a[3] = {q[0] * cs - q[1] * sn, q[0] * sn + q[1] * cs, q[2]};
    const double b[3] = {e[0] * cs - e[1] * sn, e[0] * sn + e[1] * cs, e[2]};
    const double thx = su.rot[0] * M_PI / 180, thy = su.rot[1] * M_PI / 180, thz = su.rot[2] * M_PI / 180;
    const double a1[3] = {a[0], a[1] * cos(thx) - a[2] * sin(thx), a[1] * sin(thx) + a[2] * cos(thx)};
    const double b1[3] = {b[0], b[1] * cos(thx) - b[2] * sin(thx), b[1] * sin(thx) + b[2] * cos(thx)};
    const double a2[3] = {a1[0] * cos(thy) + a1[2] * sin(thy), a1[1], -a1[0] * sin(thy) + a1[2] * cos(thy)};
    const double b2[3] = {b1[0] * cos(thy) + b1[2] * sin(thy), b1[1], -b1[0] * sin(thy) + b1[2] * cos(thy)};
    const double a3[3] = {a2[0] * cos(thz) - a2[1] * sin(thz), a2[0] * sin(thz) + a2[1] * cos(thz), a2[2]};
    const double b3[3] = {b2[0] * cos(thz) - b2[1] * sin(thz), b2[0] * sin(thz) + b2[1] * cos(thz), b2[2]};
    double* o = d.pos + ((size_t)gs * d.T + t) * 6;
    for (int i = 0; i < 3; ++i) {
        o[i] = a3[i] + su.tr[i];
        o[3 + i] = b3[i] + su.tr[i];
    }
}

// trilinear table lookup (bb_utils.cu:124-168)
__device__ double table_lookup(const BBDev& d, const BBSurfDev& su, double rr, double mach, double re, const int* br,
                               int col, int ia)
{
    const double* sect = d.sect_t + su.sect_off;
    const double* machs = d.mach_t + su.mach_off;
    const double* res = d.re_t + su.re_off;
    const double* data = d.table + su.tab_off;
    const int nm = su.nm_t, nr = su.nr_t, na = su.na_t;
    const int is1 = br[0], is2 = br[1], im1 = br[2], im2 = br[3], ir1 = br[4], ir2 = br[5];
    const double ws = is1 == is2 ? 0.5 : (rr - sect[is1]) / (sect[is2] - sect[is1]);
    const double wm = im1 == im2 ? 0.5 : (mach - machs[im1]) / (machs[im2] - machs[im1]);
    const double wr = ir1 == ir2 ? 0.5 : (re - res[ir1]) / (res[ir2] - res[ir1]);
    auto at = [&](int s, int m, int r) { return data[((((size_t)s * nm + m) * nr + r) * na + ia) * 7 + col]; };
    const double F1 = (1 - ws) * at(is1, im1, ir1) + ws * at(is2, im1, ir1);
    const double F2 = (1 - ws) * at(is1, im2, ir1) + ws * at(is2, im2, ir1);
    const double F3 = (1 - ws) * at(is1, im1, ir2) + ws * at(is2, im1, ir2);
    const double F4 = (1 - ws) * at(is1, im2, ir2) + ws * at(is2, im2, ir2);
    return (1 - wm) * (1 - wr) * F1 + wm * (1 - wr) * F2 + (1 - wm) * wr * F3 + wm * wr * F4;
}

// everything per (section, step) that does not depend on the observer or the band
__global__ void bb_prep_kernel(BBDev d)
{
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (long long)d.S * d.T) return;
    const int gs = (int)(id / d.T), t = (int)(id % d.T);
    const BBSurfDev& su = d.surf[d.secsurf[gs]];
    const int k = d.secloc[gs], ns = su.nsect, T = d.T;
    const double* geo = d.geom + 4 * (size_t)su.sec0;
    const double span = su.span;
    const double c = geo[4 * k + 3] * span;
    const double nu = 0.0000181206 / 1.22500;
    auto P = [&](int sec, int tt) { return d.pos + (((size_t)(su.sec0 + sec)) * T + tt) * 6; };
    const int tm = t == 0 ? T - 1 : t - 1, tp = t == T - 1 ? 0 : t + 1;
    const double* x0 = P(k, t);
    const double* xt = x0 + 3;
    // chordwise flow speed, Mach and Re (bb_core.cu:166-206)
    double v[3], ch[3];
    for (int i = 0; i < 3; ++i) v[i] = d.vinf[i] - (P(k, tp)[i] - P(k, tm)[i]) / (2 * d.dtau);
    for (int i = 0; i < 3; ++i) ch[i] = xt[i] - x0[i];
    const double l = sqrt(ch[0] * ch[0] + ch[1] * ch[1] + ch[2] * ch[2]);
    for (int i = 0; i < 3; ++i) ch[i] = ch[i] / l;
    const double um = v[0] * ch[0] + v[1] * ch[1] + v[2] * ch[2];
    const double mach = fabs(um / d.a0);
    const double re = fabs(um * c / nu);
    // table brackets and cl(alpha) (bb_core.cu:208-250)
    const double rr = geo[4 * k];
    int br[6];
    {
        const int is2 = count_le(d.sect_t + su.sect_off, su.ns_t, rr), im2 = count_le(d.mach_t + su.mach_off, su.nm_t, mach),
                  ir2 = count_le(d.re_t + su.re_off, su.nr_t, re);
        br[0] = max(0, is2 - 1);
        br[1] = min(is2, su.ns_t - 1);
        br[2] = max(0, im2 - 1);
        br[3] = min(im2, su.nm_t - 1);
        br[4] = max(0, ir2 - 1);
        br[5] = min(ir2, su.nr_t - 1);
    }
    const double* aoa = d.aoa_t + su.aoa_off;
    const int na = su.na_t;
    double cl[kMaxAoa];
    for (int i = 0; i < na; ++i) cl[i] = table_lookup(d, su, rr, mach, re, br, 0, i);
    int a1 = 0, a2 = 0, a3 = 0, f1 = 0, f2 = 0, f3 = 0;
    for (int i = 0; i < na; ++i) {
        if (aoa[i] >= 0.0 && !f1) { a1 = i; f1 = 1; }
        if (aoa[i] >= 6.0 && !f2) { a2 = i; f2 = 1; }
        if (cl[i] > 0 && !f3) { a3 = i; f3 = 1; }
        if (f1 && f2 && f3) break;
    }
    // indices clamped to the table so a malformed table cannot read outside it
    a1 = max(a1, 1);
    a3 = max(a3, 1);
    const double cla = (cl[a2] - cl[a1]) / (aoa[a2] - aoa[a1]);
    double w = (0 - aoa[a1 - 1]) / (aoa[a1] - aoa[a1 - 1]);
    const double cl0 = cl[a1 - 1] * (1 - w) + cl[a1] * w;
    w = (0 - cl[a3 - 1]) / (cl[a3] - cl[a3 - 1]);
    const double al0 = aoa[a3 - 1] * (1 - w) + aoa[a3] * w;
    // effective angle of attack by fixed point (bb_core.cu:291-321)
    const double* row = d.data + su.data_off + ((size_t)t * ns + k) * 7;
    const double cn = row[4], ct = row[5];
    double ae = 0.0, err = 1;
    int it = 0;
    while (err > 1e-3) {
        const double clsec = cn * cos(ae * M_PI / 180) - ct * sin(ae * M_PI / 180);
        const double ae1 = (clsec - cl0) / cla;
        err = fabs(ae1 - ae);
        ae = ae1;
        it += 1;
        if (it > 50) break;
    }
    const double alpha = fabs(ae - al0);
    // boundary-layer thicknesses (bb_core.cu:353-438)
    double bl[4];
    if (d.t_del == 0) {
        for (int i = 0; i < 4; ++i) bl[i] = row[i];
    } else if (d.t_del == 1) {
        for (int i = 0; i < na; ++i)
            if (aoa[i] >= ae) { a1 = i; break; }
        a1 = max(a1, 1);
        const double wa = (ae - aoa[a1 - 1]) / (aoa[a1] - aoa[a1 - 1]);
        for (int i = 0; i < 4; ++i) {
            const double lo = table_lookup(d, su, rr, mach, re, br, i + 3, a1 - 1);
            const double hi = table_lookup(d, su, rr, mach, re, br, i + 3, a1);
            bl[i] = c * (lo * (1 - wa) + hi * wa);
        }
    } else {
        const double lr = log10(re);
        const double d0 = c * pow(10.0, (1.6569 - 0.9045 * lr + 0.0596 * (lr * lr)));
        const double ds0 = c * pow(10.0, (3.0187 - 1.5397 * lr + 0.1059 * (lr * lr)));
        bl[1] = d0 * pow(10.0, (-0.04175 * alpha + 0.00106 * (alpha * alpha)));
        bl[3] = ds0 * pow(10.0, (-0.0432 * alpha + 0.00113 * (alpha * alpha)));
        if (alpha <= 7.5) bl[0] = d0 * pow(10.0, (0.03114 * alpha));
        else if (alpha > 12.5) bl[0] = d0 * 12.0 * pow(10.0, 0.0258 * alpha);
        else bl[0] = d0 * 0.0303 * pow(10.0, 0.2336 * alpha);
        if (alpha <= 7.5) bl[2] = ds0 * pow(10.0, (0.0679 * alpha));
        else if (alpha > 12.5) bl[2] = ds0 * 52.42 * pow(10.0, 0.0258 * alpha);
        else bl[2] = ds0 * 0.0162 * pow(10.0, 0.3066 * alpha);
    }
    // chord/span/normal frame of the section (bb_core.cu:473-513)
    const int km = k == ns - 1 ? k - 1 : k, kp = k == ns - 1 ? k : k + 1;
    double tr[3][3], n;
    for (int i = 0; i < 3; ++i) tr[0][i] = xt[i] - x0[i];
    n = sqrt(tr[0][0] * tr[0][0] + tr[0][1] * tr[0][1] + tr[0][2] * tr[0][2]);
    for (int i = 0; i < 3; ++i) tr[0][i] /= n;
    for (int i = 0; i < 3; ++i) tr[1][i] = P(kp, t)[i] - P(km, t)[i];
    n = sqrt(tr[1][0] * tr[1][0] + tr[1][1] * tr[1][1] + tr[1][2] * tr[1][2]);
    for (int i = 0; i < 3; ++i) tr[1][i] /= n;
    if (su.ccw == 1) {
        tr[2][0] = tr[0][1] * tr[1][2] - tr[0][2] * tr[1][1];
        tr[2][1] = tr[0][2] * tr[1][0] - tr[0][0] * tr[1][2];
        tr[2][2] = tr[0][0] * tr[1][1] - tr[0][1] * tr[1][0];
        n = sqrt(tr[2][0] * tr[2][0] + tr[2][1] * tr[2][1] + tr[2][2] * tr[2][2]);
        for (int i = 0; i < 3; ++i) tr[2][i] /= n;
    } else {
        tr[2][0] = tr[1][1] * tr[0][2] - tr[1][2] * tr[0][1];
        tr[2][1] = tr[1][2] * tr[0][0] - tr[1][0] * tr[0][2];
        tr[2][2] = tr[1][0] * tr[0][1] - tr[1][1] * tr[0][0];
        n = sqrt(tr[2][0] * tr[2][0] + tr[2][1] * tr[2][1] + tr[2][2] * tr[2][2]);
        // the clockwise branch divides by the square root of the norm (bb_core.cu:510-512)
        for (int i = 0; i < 3; ++i) tr[2][i] /= sqrt(n);
    }
    double ls;
    if (k == 0) ls = (geo[4 * (k + 1)] - geo[4 * k]) / 2.0 * span;
    else if (k == ns - 1) ls = (geo[4 * k] - geo[4 * (k - 1)]) / 2.0 * span;
    else ls = (geo[4 * (k + 1)] - geo[4 * (k - 1)]) / 2.0 * span;

    // band-independent scalars of core() (bb_core.cu:599-1039)
    double del_s = bl[0], del_p = bl[1], dis_s = bl[2], dis_p = bl[3];
    if (del_s < 0.0) del_s = 1.0e-10;
    if (del_p < 0.0) del_p = 1.0e-10;
    if (dis_p < 0.0) dis_p = 1.0e-10;
    if (dis_s < 0.0) dis_s = 1.0e-10;
    const double u = fabs(um), M = u / d.a0, rc = u * c / nu, mc = 0.6 * u / d.a0;
    const double rdp = u * dis_p / nu;
    const double st1 = 0.02 * pow(M, -0.6);
    double st2;
    if (alpha < 1.33) st2 = st1;
    else if (alpha > 12.5) st2 = st1 * 4.72;
    else st2 = st1 * pow(10.0, 0.0054 * ((alpha - 1.33) * (alpha - 1.33)));
    double a0r;
    if (rc < 9.52e4) a0r = 0.57;
    else if (rc > 8.57e5) a0r = 1.13;
    else a0r = (-9.57e-13) * ((rc - 8.57e5) * (rc - 8.57e5)) + 1.13;
    const double ar = (-20.0 - amin_(a0r)) / (amax_(a0r) - amin_(a0r));
    double b0r;
    if (rc < 9.52e4) b0r = 0.3;
    else if (rc > 8.57e5) b0r = 0.56;
    else b0r = (-4.48e-13) * ((rc - 8.57e5) * (rc - 8.57e5)) + 0.56;
    const double brr = (-20.0 - bmin_(b0r)) / (bmax_(b0r) - bmin_(b0r));
    double k1;
    if (rc < 2.47e5) k1 = -4.31 * log10(rc) + 156.3;
    else if (rc > 8.0e5) k1 = 128.5;
    else k1 = -9.0 * log10(rc) + 181.6;
    const double dk1 = rdp <= 5000 ? alpha * (1.43 * log10(rdp) - 5.29) : 0.0;
    const double gam = 27.094 * M + 3.31, gam0 = 23.43 * M + 4.651, bet = 72.65 * M + 10.74, bet0 = -34.19 * M - 13.82;
    double k2;
    if (alpha < gam0 - gam) k2 = k1 - 1000.0;
    else if (alpha > gam0 + gam) k2 = k1 - 12.0;
    else k2 = k1 + sqrt(bet * bet - (bet / gam) * (bet / gam) * ((alpha - gam0) * (alpha - gam0))) + bet0;
    const bool stall = (alpha >= gam0 || alpha > 12.5);
    double ars = 0.0, k2s = 0.0;
    if (stall) {
        const double rcn = 3.0 * rc;
        double a0n;
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
        ars = (-20.0 - amin_(a0n)) / (amax_(a0n) - amin_(a0n));
    }
    const double m5 = pow(M, 5);
    // LBL-VS (bb_core.cu:863-915)
    double stpk = 1.0, g23 = 0.0;
    const int trip0 = su.trip == 0;
    if (trip0) {
        double stl;
        if (rc < 1.3e5) stl = 0.18;
        else if (rc > 1.3e5 && rc <= 4e5) stl = 0.001756 * pow(rc, 0.3931);
        else stl = 0.28;
        stpk = pow(10.0, (-0.04 * alpha)) * stl;
        const double rc0 = alpha <= 3.0 ? pow(10.0, (0.215 * alpha + 4.978)) : pow(10.0, (0.120 * alpha + 5.263));
        const double dd = rc / rc0;
        double g2;
        if (dd <= 0.3237) g2 = 77.852 * log10(dd) + 15.328;
        else if (dd <= 0.5689) g2 = 65.188 * log10(dd) + 9.125;
        else if (dd <= 1.7579) g2 = -114.052 * (log10(dd) * log10(dd));
        else if (dd <= 3.0889) g2 = -65.188 * log10(dd) + 9.125;
        else g2 = -77.852 * log10(dd) + 15.328;
        g23 = g2 + (171.04 - 3.03 * alpha);
    }
    // TEB-VS, h = 0.5 mm, psi = 14 deg (bb_core.cu:917-971)
    const double h = 0.0005, psiv = 14.0;
    const double hd = h / ((dis_s + dis_p) / 2.0), dh_ = 1.0 / hd;
    const double aterm = 0.212 - 0.0045 * psiv;
    const double stpeak =
        hd >= 0.2 ? aterm / (1.0 + 0.235 * dh_ - 0.0132 * (dh_ * dh_)) : 0.1 * hd + 0.095 - 0.00243 * psiv;
    const double g4 = hd <= 5.0 ? 17.5 * log10(hd) + 157.5 - 1.114 * psiv : 169.7 - 1.114 * psiv;
    const double hdp = 6.724 * (hd * hd) - 4.019 * hd + 1.107;
    // tip vortex on the last section (bb_core.cu:975-1039)
    const int tip = k == ns - 1;
    double tl = 1.0, umm = 1.0, gtip = 0.0;
    if (tip) {
        const double ar0[6] = {2.0, 2.67, 4.0, 6.0, 12.0, 24.0};
        const double rat0[6] = {0.54, 0.62, 0.71, 0.79, 0.89, 0.95};
        const double AR = span / c;
        double rat;
        if (AR < ar0[0]) rat = rat0[0];
        else if (AR > ar0[5]) rat = rat0[5];
        else {
            int kk = 0;
            while (kk < 5 && !(AR < ar0[kk])) kk++;
            kk = max(kk, 1);
            rat = rat0[kk - 1] * (ar0[kk] - AR) / (ar0[kk] - ar0[kk - 1]) +
                  rat0[kk] * (AR - ar0[kk - 1]) / (ar0[kk] - ar0[kk - 1]);
        }
        const double at = alpha * rat;
        tl = fabs(at) <= 2.0 ? (0.023 + 0.0169 * at) * c : (0.0378 + 0.0095 * at) * c;
        const double mm = (1.0 + 0.036 * at) * M;
        umm = mm * d.a0;
        gtip = M * M * (mm * mm * mm) * (tl * tl);
    }

    float* g = d.geo + id * kGeo;
    g[0] = (float)xt[0]; g[1] = (float)xt[1]; g[2] = (float)xt[2];
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) g[3 + 3 * a + b] = (float)tr[a][b];
    g[12] = (float)M; g[13] = (float)mc; g[14] = stall ? 1.f : 0.f; g[15] = 0.f;
    float* q = d.sc + id * kSc;
    q[0] = (float)u; q[1] = (float)M; q[2] = (float)mc; q[3] = (float)dis_s; q[4] = (float)dis_p;
    q[5] = (float)del_p; q[6] = (float)ls; q[7] = (float)st1; q[8] = (float)st2; q[9] = (float)ar;
    q[10] = (float)brr; q[11] = (float)(k1 - 3.0); q[12] = (float)dk1; q[13] = (float)k2; q[14] = stall ? 1.f : 0.f;
    q[15] = (float)ars; q[16] = (float)k2s; q[17] = (float)trip0; q[18] = (float)stpk; q[19] = (float)g23;
    q[20] = (float)hd; q[21] = (float)stpeak; q[22] = (float)g4; q[23] = (float)hdp; q[24] = (float)tip;
    q[25] = (float)tl; q[26] = (float)umm; q[27] = (float)gtip;
    q[28] = (float)(dis_p * m5 * ls); q[29] = (float)(dis_s * m5 * ls); q[30] = (float)(del_p * m5 * ls);
    q[31] = (float)(pow(M, 5.5) * h * ls);
}

// spectral amplitudes per (section, step, band), FP32 (bb_core.cu:637-1039)
__global__ void bb_spec_kernel(const float* __restrict__ sc, const double* __restrict__ ff, float* __restrict__ amp,
                               long long nst)
{
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nst * kBands) return;
    const long long st = id / kBands;
    const int fb = (int)(id % kBands);
    const float* q = sc + st * kSc;
    const float f = (float)ff[fb];
    const float u = q[0];
    const float sts = f * q[3] / u, stp = f * q[4] / u;
    // TBL-TE pressure and suction sides
    const float as = fabsf(log10f(sts / q[7])), ap = fabsf(log10f(stp / q[7]));
    const float aas = amin_(as) + q[9] * (amax_(as) - amin_(as));
    const float aap = amin_(ap) + q[9] * (amax_(ap) - amin_(ap));
    const float Ap = q[28] * exp10f((aap + q[11] + q[12]) * 0.1f);
    const float As = q[29] * exp10f((aas + q[11]) * 0.1f);
    // separation (angle-of-attack) contribution
    float Aa;
    const float b = fabsf(log10f(sts / q[8]));
    if (q[14] != 0.f) Aa = q[29] * exp10f((amin_(b) + q[15] * (amax_(b) - amin_(b)) + q[16]) * 0.1f);
    else Aa = q[29] * exp10f((bmin_(b) + q[10] * (bmax_(b) - bmin_(b)) + q[13]) * 0.1f);
    // LBL-VS
    float Al = 0.f;
    if (q[17] != 0.f) {
        const float e = (f * q[5] / u) / q[18], le = log10f(e);
        float g1;
        if (e <= 0.5974f) g1 = 39.8f * le - 11.12f;
        else if (e <= 0.8545f) g1 = 98.409f * le + 2.0f;
        else if (e <= 1.17f) g1 = -5.076f + sqrtf(2.484f - 506.25f * (le * le));
        else if (e <= 1.674f) g1 = -98.409f * le + 2.0f;
        else g1 = -39.80f * le - 11.12f;
        Al = q[30] * exp10f((g1 + q[19]) * 0.1f);
    }
    // TEB-VS
    const float eta = log10f((f * 0.0005f / u) / q[21]);
    const float g514 = g5_(q[20], eta), g50 = g5_(q[23], eta);
    float g5 = g50 + 0.0714f * 14.0f * (g514 - g50);
    if (g5 > 0.f) g5 = 0.f;
    const float f4 = g5_(0.25f, eta);
    if (g5 > f4) g5 = f4;
    const float At = q[31] * exp10f((q[22] + g5) * 0.1f);
    // tip vortex
    float Av = 0.f;
    if (q[24] != 0.f) {
        const float lg = log10f(f * q[25] / q[26]) + 0.3f;
        Av = exp10f((126.0f - 30.5f * (lg * lg)) * 0.1f);
    }
    // band pairs interleaved: [item][band / 2][field][band % 2] (the operand pairs of the
    // packed contraction in bb_obs_kernel)
    float* o = amp + st * (kBands * kAmp) + (size_t)(fb >> 1) * (2 * kAmp) + (fb & 1);
    const float v[kAmp] = {Ap, As, Aa, Al, At, Av, q[27], 0.f};
#pragma unroll
    for (int c = 0; c < kAmp; ++c) o[2 * c] = v[c];
}

// Observer contraction.  Block = 64 observers (lane l serves observers l and l + 32) x
// 21 warps, one per pair of bands.  Per tile of kTI (section, step) items, the amplitudes
// of all 42 bands (contiguous in `amp`, 1344 B per item, band pairs interleaved) and the
// items' geometry records arrive in shared memory by one bulk copy into a ring of three
// buffers (two tiles ahead of the one consumed); the directivity factors D of the block's
// observers are computed into shared memory one tile ahead (double-buffered, each stored
// twice, as the operand pair of a packed instruction), in the same phase as the current
// tile's sums, so that one block barrier per tile separates the phases; each lane adds,
// for its two observers and its warp's two bands, the clipped energies of every item in
// packed FP32 (one f32x2 operation covers both bands).  The amplitude reads are warp-uniform (shared-
// memory broadcasts), the D reads conflict-free.  FP32 partial sums over at most 1024
// items are folded into FP64 sums private to the block's (observer tile, item range):
// part[split][band][component][observer], reduced over the splits by bb_final_kernel.
constexpr int kObsPerLane = 2;
constexpr int kObsBlock = 32 * kObsPerLane;  // 64
constexpr int kPairWarps = kBands / 2;       // 21
constexpr int kBpmThreads = 32 * kPairWarps; // 672
constexpr int kTI = 32;                      // items per tile
constexpr int kFoldTiles = 32;               // 1024 items per FP32 partial
constexpr int kAmpItemBytes = kBands * kAmp * 4;  // 1344
constexpr int kGeoItemBytes = kGeo * 4;           // 64
static_assert(kBands % 2 == 0, "band pairs");
static_assert(kAmpItemBytes % 16 == 0 && kGeoItemBytes % 16 == 0, "bulk copy granularity");

// dynamic shared memory of bb_obs_kernel: kObsRing x (amplitude tile + geometry tile), 2 D
// tiles (float4 (Dh, Dh, Dl, Dl) per item and observer), the block's observers, kObsRing
// mbarriers
constexpr int kObsRing = 3;
constexpr size_t kObsSmemA = (size_t)kTI * kAmpItemBytes;
constexpr size_t kObsSmemG = (size_t)kTI * kGeoItemBytes;
constexpr size_t kObsSmemBuf = kObsSmemA + kObsSmemG;
constexpr size_t kObsSmemD = (size_t)kTI * kObsBlock * sizeof(float4);
constexpr size_t kObsSmem =
    kObsRing * kObsSmemBuf + 2 * kObsSmemD + kObsBlock * 3 * sizeof(float) + kObsRing * sizeof(uint64_t);

__device__ __forceinline__ float2 bb_directivity(const float* geo, const float* obs, int o, float vx, float vy,
                                                 float vz, float aa, float iaMv)
{
    const float4* g = reinterpret_cast<const float4*>(geo);
    const float4 g0 = g[0], g1 = g[1], g2 = g[2], g3 = g[3];
    float rx = obs[3 * o] - g0.x, ry = obs[3 * o + 1] - g0.y, rz = obs[3 * o + 2] - g0.z;
    // convected emission time (bb_core.cu:515-520)
    const float bb = rx * vx + ry * vy + rz * vz;
    const float cc = rx * rx + ry * ry + rz * rz;
    const float tau = (-bb + sqrtf(bb * bb + aa * cc)) * iaMv;
    rx -= vx * tau;
    ry -= vy * tau;
    rz -= vz * tau;
    const float r2 = rx * rx + ry * ry + rz * rz;
    // frame rows: chord (g0.w, g1.x, g1.y), span (g1.z, g1.w, g2.x), normal (g2.y, g2.z, g2.w)
    const float p0 = rx * g0.w + ry * g1.x + rz * g1.y;
    const float p1 = rx * g1.z + ry * g1.w + rz * g2.x;
    const float p2 = rx * g2.y + ry * g2.z + rz * g2.w;
    const float cx = fabsf(p0) * rsqrtf(r2);                // cos(theta)
    const float cy = fabsf(p1) * rsqrtf(p1 * p1 + p2 * p2);  // cos(phi)
    // sin^2(theta/2), sin^2(theta), sin^2(phi) without the acos; a zero angle is replaced
    // by 1e-10 as the reference does (bb_core.cu:525-530)
    const float sh2 = cx >= 1.f ? 2.5e-21f : 0.5f * (1.f - cx);
    const float sth2 = cx >= 1.f ? 1e-20f : (1.f - cx) * (1.f + cx);
    const float sp2 = cy >= 1.f ? 1e-20f : (1.f - cy) * (1.f + cy);
    // directivities d_h, d_l (bb_core.cu:620-624) over r^2
    const float M = g3.x, Mc = g3.y;
    const float q1 = 1.f + M * cx, q2 = 1.f + (M - Mc) * cx;
    const float Dh = __fdividef(2.f * sh2 * sp2, q1 * q2 * q2 * r2);
    const float Dl = __fdividef(sth2 * sp2, q1 * q1 * q1 * q1 * r2);
    return make_float2(Dh, g3.z != 0.f ? Dl : Dh);
}

__device__ __forceinline__ float2 clip2(float2 v, float lo) { return make_float2(fmaxf(v.x, lo), fmaxf(v.y, lo)); }

__global__ void __launch_bounds__(kBpmThreads, 1) bb_obs_kernel(const float* __restrict__ geo,
                                                                const float* __restrict__ amp,
                                                                const float* __restrict__ obs, int O, long long nst,
                                                                long long per_split, float vx, float vy, float vz,
                                                                float a0, int aa_mode, double* __restrict__ part,
                                                                DeviceErr* err)
{
    extern __shared__ __align__(128) unsigned char sm[];
    float4* sD0 = reinterpret_cast<float4*>(sm + kObsRing * kObsSmemBuf);  // 2 x [kTI][kObsBlock]
    float* sObs = reinterpret_cast<float*>(sm + kObsRing * kObsSmemBuf + 2 * kObsSmemD);
    uint64_t* bars =
        reinterpret_cast<uint64_t*>(sm + kObsRing * kObsSmemBuf + 2 * kObsSmemD + kObsBlock * 3 * sizeof(float));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;  // warp = band pair
    const int o0 = blockIdx.x * kObsBlock;
    const long long st_begin = (long long)blockIdx.y * per_split;
    const long long st_end = min(nst, st_begin + per_split);
    const int ntiles = st_end > st_begin ? (int)((st_end - st_begin + kTI - 1) / kTI) : 0;
    const float aMv = a0 * a0 - (vx * vx + vy * vy + vz * vz);
    const float aa = aa_mode == 1 ? 0.f : aMv;
    const float iaMv = 1.0f / aMv;
    double* mine = part + (size_t)blockIdx.y * kBands * 6 * O;  // [band][component][observer]

    for (int i = threadIdx.x; i < kObsBlock * 3; i += blockDim.x) {
        const int o = o0 + i / 3;
        sObs[i] = o < O ? obs[3 * o0 + i] : 0.f;
    }
    if (threadIdx.x == 0) {
        for (int b = 0; b < kObsRing; ++b) mbar_init(&bars[b], 1);
        mbar_fence_init();
    }
    __syncthreads();
    // tile j -> buffer j % kObsRing (phase j / kObsRing of its barrier): amplitudes, then
    // the geometry of its items
    auto tile_n = [&](int j) { return (int)min((long long)kTI, st_end - (st_begin + (long long)j * kTI)); };
    auto buf_of = [&](int j) { return sm + (size_t)(j % kObsRing) * kObsSmemBuf; };
    auto issue = [&](int j) {
        const long long t0 = st_begin + (long long)j * kTI;
        const int n = tile_n(j);
        unsigned char* buf = buf_of(j);
        mbar_expect_tx(&bars[j % kObsRing], (uint32_t)(n * (kAmpItemBytes + kGeoItemBytes)));
        bulk_g2s(buf, amp + t0 * kBands * kAmp, (uint32_t)(n * kAmpItemBytes), &bars[j % kObsRing]);
        bulk_g2s(buf + kObsSmemA, geo + t0 * kGeo, (uint32_t)(n * kGeoItemBytes), &bars[j % kObsRing]);
    };
    auto wait_tile = [&](int j) {
        return mbar_wait_bounded(&bars[j % kObsRing], (uint32_t)((j / kObsRing) & 1));
    };
    // D of every (item, observer) of tile j (bb_core.cu:515-530, 620-624) into D buffer j & 1
    auto directivity = [&](int j) {
        const int n = tile_n(j);
        const float* sG = reinterpret_cast<const float*>(buf_of(j) + kObsSmemA);
        float4* sD = sD0 + (size_t)(j & 1) * kTI * kObsBlock;
#pragma unroll 1
        for (int pidx = threadIdx.x; pidx < kTI * kObsBlock; pidx += blockDim.x) {
            const int it = pidx / kObsBlock, ol = pidx % kObsBlock;
            float2 D = make_float2(0.f, 0.f);
            if (it < n && o0 + ol < O) D = bb_directivity(sG + it * kGeo, sObs, ol, vx, vy, vz, aa, iaMv);
            sD[it * kObsBlock + ol] = make_float4(D.x, D.x, D.y, D.y);
        }
    };
    int issued = 0;
    if (threadIdx.x == 0)
        for (; issued < kObsRing && issued < ntiles; ++issued) issue(issued);

    float2 acc[kObsPerLane][6];  // (band 2 warp, band 2 warp + 1)
#pragma unroll
    for (int q = 0; q < kObsPerLane; ++q)
#pragma unroll
        for (int c = 0; c < 6; ++c) acc[q][c] = make_float2(0.f, 0.f);
    auto fold = [&]() {
#pragma unroll
        for (int q = 0; q < kObsPerLane; ++q) {
            const int o = o0 + q * 32 + lane;
            if (o < O) {
                // addresses formed here, not hoisted out of the item loop
                size_t stride = (size_t)O;
                asm volatile("" : "+l"(stride));
                double* p0 = mine + (size_t)(2 * warp) * 6 * stride + o;  // band 2 warp
                double* p1 = p0 + 6 * stride;                             // band 2 warp + 1
#pragma unroll
                for (int c = 0; c < 6; ++c) {
                    p0[c * stride] += (double)acc[q][c].x;
                    p1[c * stride] += (double)acc[q][c].y;
                }
            }
#pragma unroll
            for (int c = 0; c < 6; ++c) acc[q][c] = make_float2(0.f, 0.f);
        }
    };
    int aborted_at = -1;
    if (ntiles > 0) {
        const bool ok = wait_tile(0);
        if (ok) directivity(0);
        if (__syncthreads_or(!ok)) aborted_at = 0;
    }
    int tiles = 0;
    for (int j = 0; j < ntiles && aborted_at < 0; ++j) {
        // the next tile's D, in the same phase as this tile's sums
        bool ok = true;
        if (j + 1 < ntiles) {
            ok = wait_tile(j + 1);
            if (ok) directivity(j + 1);
        }
        const int n = tile_n(j);
        const float4* sA = reinterpret_cast<const float4*>(buf_of(j));
        const float4* sD = sD0 + (size_t)(j & 1) * kTI * kObsBlock;
#pragma unroll 1
        for (int it = 0; it < n; ++it) {
            // the warp's band pair: fields (Ap, As), (Aa, Al), (At, Av), (gtip, -) of both bands
            const float4* a = sA + (it * kPairWarps + warp) * 4;
            const float4 a0v = a[0], a1v = a[1], a2v = a[2], a3v = a[3];
            const float2 Ap = make_float2(a0v.x, a0v.y), As = make_float2(a0v.z, a0v.w);
            const float2 Aa = make_float2(a1v.x, a1v.y), Al = make_float2(a1v.z, a1v.w);
            const float2 At = make_float2(a2v.x, a2v.y), Av = make_float2(a2v.z, a2v.w);
            const float2 Ag = make_float2(a3v.x, a3v.y);
            const bool tip = Av.x != 0.f || Av.y != 0.f;
#pragma unroll
            for (int q = 0; q < kObsPerLane; ++q) {
                const float4 D = sD[it * kObsBlock + q * 32 + lane];
                const float2 Dh = make_float2(D.x, D.y), Dl = make_float2(D.z, D.w);
                acc[q][0] = add2(acc[q][0], clip2(mul2(Dh, Ap), 1e-10f));  // TBL-TE pressure side
                acc[q][1] = add2(acc[q][1], clip2(mul2(Dh, As), 1e-10f));  // TBL-TE suction side
                acc[q][2] = add2(acc[q][2], clip2(mul2(Dl, Aa), 1e-10f));  // separation
                acc[q][3] = fma2(Dh, Al, acc[q][3]);                       // LBL-VS
                acc[q][4] = fma2(Dh, At, acc[q][4]);                       // TEB-VS
                if (tip) acc[q][5] = fma2(Av, clip2(mul2(Dh, Ag), 2.2204460492503131e-16f), acc[q][5]);  // tip
            }
        }
        // every thread is done with tile j's buffer and D tile, and tile j + 1's D is
        // complete: refill the buffer with tile j + kObsRing
        if (__syncthreads_or(!ok)) {
            aborted_at = j + 1;
            break;
        }
        if (threadIdx.x == 0 && j + kObsRing < ntiles) issue(issued++);
        if (++tiles == kFoldTiles) {
            fold();
            tiles = 0;
        }
    }
    if (aborted_at >= 0) {
        // wait (bounded) for the copies still in flight (tiles aborted_at .. issued - 1,
        // counted by thread 0, which issues them) before the block exits
        if (threadIdx.x == 0) {
            flag(err, ACUM_DEVERR_TIMEOUT, &err->timeout);
            for (int j = aborted_at; j < issued; ++j) (void)wait_tile(j);
        }
        __syncthreads();
        return;
    }
    fold();
}

// Energy mean over steps and band sum in dB (bb_core.cu:563-583); the component sums
// of the clipped energies become the seven levels.  Components of `sums`: TBL pressure,
// suction, separation, LBL, TEB, tip; of BBspl: total, separation, suction, pressure,
// LBL, TEB, tip.
// one thread per (band, observer), observers consecutive (coalesced reads of the sums):
// the band's seven component levels
__global__ void bb_final_kernel(const double* __restrict__ part, int nsplit, int O, int T,
                                const double* __restrict__ seed_spl, double* __restrict__ spl)
{
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (long long)O * kBands) return;
    const int f = (int)(idx / O), o = (int)(idx % O);
    {
        double s[6];
        for (int c = 0; c < 6; ++c) {
            double v = 0.0;
            for (int k = 0; k < nsplit; ++k) v += part[(((size_t)k * kBands + f) * 6 + c) * O + o];
            s[c] = v;
        }
        // the -100 dB seed of every (observer, step, band, component) contributes T * 1e-10
        const double floor_t = T * 1e-10;
        const double comp[7] = {s[0] + s[1] + s[2] + s[3] + s[4] + s[5], s[2], s[1], s[0], s[3], s[4], s[5]};
        double* out = spl + ((size_t)o * kBands + f) * 7;
        const double* seed = seed_spl + ((size_t)o * kBands + f) * 7;
        for (int c = 0; c < 7; ++c) out[c] = 10.0 * log10((pow(10.0, seed[c] / 10.0) + floor_t + comp[c]) / (double)T);
    }
}

// one thread per observer: the OASPL, the band totals summed in band order
__global__ void bb_oaspl_kernel(int O, const double* __restrict__ seed_oas, const double* __restrict__ spl,
                                double* __restrict__ oaspl)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= O) return;
    double oas = pow(10.0, seed_oas[o] / 10.0);
    for (int f = 0; f < kBands; ++f) oas += pow(10.0, spl[((size_t)o * kBands + f) * 7] / 10.0);
    oaspl[o] = 10.0 * log10(oas);
}

// ---------------------------------------------------------------- host side

static int bpm_upload(acum_ctx* ctx)
{
    BpmState* s = state(ctx);
    const BBDeck& bb = ctx->bb;
    const int nbb = bb.nsurf;
    std::vector<BBSurfDev> sd(nbb);
    std::vector<int> secsurf, secloc;
    int sec = 0, so = 0, ao = 0, mo = 0, ro = 0;
    long long dofs = 0, tofs = 0;
    for (int i = 0; i < nbb; ++i) {
        BBSurfDev& d = sd[i];
        d.span = bb.span[i];
        d.omega = bb.omega[i];
        d.psi_off = bb.psi_offset[i];
        for (int c = 0; c < 3; ++c) {
            d.rot[c] = bb.rotate[3 * i + c];
            d.tr[c] = bb.translate[3 * i + c];
        }
        d.ccw = bb.ccw[i];
        d.trip = bb.trip[i];
        d.nsect = bb.nsect[i];
        d.sec0 = sec;
        d.data_off = dofs;
        d.ns_t = bb.ns_t[i];
        d.na_t = bb.na_t[i];
        d.nm_t = bb.nm_t[i];
        d.nr_t = bb.nr_t[i];
        if (d.na_t > kMaxAoa) return fail(ctx, ACUM_ERR_UNSUPPORTED, "broadband tables with more than 64 AoA entries");
        if (d.nsect < 3) return fail(ctx, ACUM_ERR_INVALID, "a broadband surface needs at least 3 sections");
        d.sect_off = so;
        d.aoa_off = ao;
        d.mach_off = mo;
        d.re_off = ro;
        d.tab_off = tofs;
        for (int k = 0; k < d.nsect; ++k) {
            secsurf.push_back(i);
            secloc.push_back(k);
        }
        sec += d.nsect;
        dofs += (long long)ctx->T * d.nsect * 7;
        so += d.ns_t;
        ao += d.na_t;
        mo += d.nm_t;
        ro += d.nr_t;
        tofs += (long long)d.ns_t * d.nm_t * d.nr_t * d.na_t * 7;
    }
    s->S = sec;
    s->nbb = nbb;
    s->T = ctx->T;
    auto up = [&](DBuf<double>& b, const std::vector<double>& v) -> cudaError_t {
        cudaError_t e = b.ensure(std::max<size_t>(v.size(), 1));
        if (e != cudaSuccess) return e;
        return cudaMemcpy(b.p, v.data(), v.size() * 8, cudaMemcpyHostToDevice);
    };
    cudaError_t e;
    if ((e = s->surf.ensure(nbb)) != cudaSuccess) return cuda_fail(ctx, e, "bpm alloc");
    if ((e = cudaMemcpy(s->surf.p, sd.data(), nbb * sizeof(BBSurfDev), cudaMemcpyHostToDevice)) != cudaSuccess)
        return cuda_fail(ctx, e, "bpm upload");
    if ((e = s->secsurf.ensure(sec)) != cudaSuccess || (e = s->secloc.ensure(sec)) != cudaSuccess)
        return cuda_fail(ctx, e, "bpm alloc");
    cudaMemcpy(s->secsurf.p, secsurf.data(), sec * 4, cudaMemcpyHostToDevice);
    cudaMemcpy(s->secloc.p, secloc.data(), sec * 4, cudaMemcpyHostToDevice);
    if ((e = up(s->geom, bb.geom)) != cudaSuccess || (e = up(s->data, bb.data)) != cudaSuccess ||
        (e = up(s->sect_t, bb.sect_t)) != cudaSuccess || (e = up(s->aoa_t, bb.aoa_t)) != cudaSuccess ||
        (e = up(s->mach_t, bb.mach_t)) != cudaSuccess || (e = up(s->re_t, bb.re_t)) != cudaSuccess ||
        (e = up(s->table, bb.table)) != cudaSuccess)
        return cuda_fail(ctx, e, "bpm upload");
    std::vector<double> ff(kBandHz, kBandHz + kBands);
    if ((e = up(s->ff, ff)) != cudaSuccess) return cuda_fail(ctx, e, "bpm upload");
    const size_t nst = (size_t)sec * ctx->T;
    if ((e = s->pos.ensure(nst * 6)) != cudaSuccess || (e = s->geo.ensure(nst * kGeo)) != cudaSuccess ||
        (e = s->sc.ensure(nst * kSc)) != cudaSuccess || (e = s->amp.ensure(nst * kBands * kAmp)) != cudaSuccess)
        return cuda_fail(ctx, e, "bpm alloc");
    s->uploaded = true;
    ctx->bb_dirty = false;
    return ACUM_OK;
}

// Runs the broadband path on the context's deck; seeds (dB) may be null (-100 dB).
static int bpm_run(acum_ctx* ctx, int aa_mode, const double* seed_spl_h, const double* seed_oas_h, double* spl_h,
                   double* oas_h)
{
    if (!ctx->have_deck || !ctx->have_bb) return fail(ctx, ACUM_ERR_STATE, "no broadband deck");
    if (aa_mode != 0 && aa_mode != 1) return fail(ctx, ACUM_ERR_INVALID, "aa_mode must be 0 or 1");
    DeviceGuard g(ctx->device);
    BpmState* s = state(ctx);
    if (ctx->bb_dirty || !s->uploaded) {
        int rc = bpm_upload(ctx);
        if (rc) return rc;
    }
    const int O = ctx->nobs, T = ctx->T;
    const long long nst = (long long)s->S * T;
    cudaStream_t st = ctx->stream;
    cudaError_t e;
    if ((e = s->spl.ensure((size_t)O * kBands * 7)) != cudaSuccess || (e = s->oaspl.ensure(O)) != cudaSuccess ||
        (e = s->seed_spl.ensure((size_t)O * kBands * 7)) != cudaSuccess || (e = s->seed_oas.ensure(O)) != cudaSuccess)
        return cuda_fail(ctx, e, "bpm alloc");
    std::vector<double> sspl((size_t)O * kBands * 7, -100.0), soas(O, -100.0);
    if (seed_spl_h) memcpy(sspl.data(), seed_spl_h, sspl.size() * 8);
    if (seed_oas_h) memcpy(soas.data(), seed_oas_h, soas.size() * 8);
    cudaMemcpyAsync(s->seed_spl.p, sspl.data(), sspl.size() * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(s->seed_oas.p, soas.data(), soas.size() * 8, cudaMemcpyHostToDevice, st);
    BBDev d;
    d.surf = s->surf.p;
    d.secsurf = s->secsurf.p;
    d.secloc = s->secloc.p;
    d.geom = s->geom.p;
    d.data = s->data.p;
    d.sect_t = s->sect_t.p;
    d.aoa_t = s->aoa_t.p;
    d.mach_t = s->mach_t.p;
    d.re_t = s->re_t.p;
    d.table = s->table.p;
    d.pos = s->pos.p;
    d.geo = s->geo.p;
    d.sc = s->sc.p;
    d.S = s->S;
    d.T = T;
    d.dtau = ctx->der.dTau;
    d.a0 = ctx->in.a0;
    for (int c = 0; c < 3; ++c) d.vinf[c] = ctx->der.vinf[c];
    d.t_del = ctx->bb.t_del;
    const int nb = (int)((nst + 127) / 128);
    cudaEventRecord(ctx->ev[EV_BPM0], st);
    bb_pos_kernel<<<nb, 128, 0, st>>>(d);
    bb_prep_kernel<<<nb, 128, 0, st>>>(d);
    bb_spec_kernel<<<(int)((nst * kBands + 255) / 256), 256, 0, st>>>(s->sc.p, s->ff.p, s->amp.p, nst);
    // item ranges: the number of splits (up to 8 waves of resident blocks) with the
    // smallest wave-quantisation loss
    const int oblocks = (O + kObsBlock - 1) / kObsBlock;
    static bool configured = false;
    if (!configured) {
        if ((e = cudaFuncSetAttribute(bb_obs_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kObsSmem)) !=
            cudaSuccess)
            return cuda_fail(ctx, e, "bpm configure");
        configured = true;
    }
    int per_sm = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, bb_obs_kernel, kBpmThreads, kObsSmem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    const int slots = per_sm * ctx->num_sms;
    int split = 1;
    double best = 1e30;
    const int maxs = (int)std::max<long long>(1, std::min<long long>((8 * slots + oblocks - 1) / oblocks,
                                                                      (nst + kTI - 1) / kTI));
    for (int k = 1; k <= maxs; ++k) {
        const double waves = (double)oblocks * k / slots;
        const double cost = std::ceil(waves) / waves + 0.01 * k;
        if (cost < best) {
            best = cost;
            split = k;
        }
    }
    const long long per_split = ((nst + split - 1) / split + kTI - 1) / kTI * kTI;
    split = (int)((nst + per_split - 1) / per_split);
    if ((e = s->sums.ensure((size_t)split * kBands * 6 * O)) != cudaSuccess) return cuda_fail(ctx, e, "bpm alloc");
    cudaMemsetAsync(s->sums.p, 0, (size_t)split * kBands * 6 * O * 8, st);
    dim3 grid(oblocks, split);
    cudaEventRecord(ctx->ev[EV_BOBS0], st);
    bb_obs_kernel<<<grid, kBpmThreads, kObsSmem, st>>>(s->geo.p, s->amp.p, ctx->d_obs32.p, O, nst, per_split,
                                                       (float)d.vinf[0], (float)d.vinf[1], (float)d.vinf[2],
                                                       (float)d.a0, aa_mode, s->sums.p, ctx->d_err.p);
    cudaEventRecord(ctx->ev[EV_BOBS1], st);
    bb_final_kernel<<<(int)(((long long)O * kBands + 127) / 128), 128, 0, st>>>(s->sums.p, split, O, T,
                                                                              s->seed_spl.p, s->spl.p);
    bb_oaspl_kernel<<<(O + 127) / 128, 128, 0, st>>>(O, s->seed_oas.p, s->spl.p, s->oaspl.p);
    cudaEventRecord(ctx->ev[EV_BPM1], st);
    ctx->launches += 6;
    ctx->bpm_timed = true;
    if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(ctx, e, "bpm launch");
    ctx->h_spl.resize((size_t)O * kBands * 7);
    ctx->h_oaspl.resize(O);
    cudaMemcpyAsync(ctx->h_spl.data(), s->spl.p, ctx->h_spl.size() * 8, cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(ctx->h_oaspl.data(), s->oaspl.p, O * 8, cudaMemcpyDeviceToHost, st);
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(ctx, e, "bpm run");
    {
        DeviceErr h;
        if ((e = cudaMemcpy(&h, ctx->d_err.p, sizeof(h), cudaMemcpyDeviceToHost)) != cudaSuccess)
            return cuda_fail(ctx, e, "bpm error word");
        if (h.bits & ACUM_DEVERR_TIMEOUT) {
            cudaMemset(ctx->d_err.p, 0, sizeof(DeviceErr));
            return fail(ctx, ACUM_ERR_TIMEOUT, "a bounded shared-memory pipeline wait ran out; results are incomplete");
        }
    }
    if (spl_h) memcpy(spl_h, ctx->h_spl.data(), ctx->h_spl.size() * 8);
    if (oas_h) memcpy(oas_h, ctx->h_oaspl.data(), O * 8);
    ctx->have_bpm = true;
    return ACUM_OK;
}

}  // namespace acum

using namespace acum;

extern "C" int acum_set_bb(acum_ctx* ctx, const acum_bb_desc* b)
{
    acum::NvtxRange nvtx_range_("acum_set_bb");
    if (!ctx || !b) return fail(ctx, ACUM_ERR_INVALID, "acum_set_bb: null argument");
    if (!ctx->have_deck) return fail(ctx, ACUM_ERR_STATE, "acum_set_bb: set the tonal deck first");
    if (b->nsurf <= 0 || b->nsurf > ctx->nsurf)
        return fail(ctx, ACUM_ERR_INVALID,
                    "Number of surfaces considered for broadband noise cannot be higher than the available surfaces");
    BBDeck bb;
    const int n = b->nsurf, T = ctx->T;
    bb.nsurf = n;
    bb.t_del = b->t_del;
    bb.span.assign(b->span, b->span + n);
    bb.omega.assign(b->omega, b->omega + n);
    bb.psi_offset.assign(b->psi_offset, b->psi_offset + n);
    bb.rotate.assign(b->rotate, b->rotate + 3 * n);
    bb.translate.assign(b->translate, b->translate + 3 * n);
    bb.ccw.assign(b->ccw, b->ccw + n);
    bb.trip.assign(b->trip, b->trip + n);
    bb.nsect.assign(b->nsect, b->nsect + n);
    size_t ns = 0, nt = 0, na = 0, nm = 0, nr = 0, ntab = 0;
    for (int i = 0; i < n; ++i) {
        if (b->nsect[i] < 3) return fail(ctx, ACUM_ERR_INVALID, "a broadband surface needs at least 3 sections");
        ns += b->nsect[i];
        nt += b->ns_t[i];
        na += b->na_t[i];
        nm += b->nm_t[i];
        nr += b->nr_t[i];
        ntab += (size_t)b->ns_t[i] * b->na_t[i] * b->nm_t[i] * b->nr_t[i] * 7;
    }
    bb.geom.assign(b->geom, b->geom + 4 * ns);
    bb.data.assign(b->data, b->data + (size_t)T * ns * 7);
    // cn, cc divided by (r/R)^2 for rotating surfaces, as read_BB_inputs does (io.cu:509-512)
    size_t so = 0, dof = 0;
    for (int i = 0; i < n; ++i) {
        if ((float)bb.omega[i] != 0.0f)
            for (int t = 0; t < T; ++t)
                for (int k = 0; k < b->nsect[i]; ++k) {
                    const double rr = bb.geom[4 * (so + k)];
                    bb.data[dof + ((size_t)t * b->nsect[i] + k) * 7 + 4] /= rr * rr;
                    bb.data[dof + ((size_t)t * b->nsect[i] + k) * 7 + 5] /= rr * rr;
                }
        so += b->nsect[i];
        dof += (size_t)T * b->nsect[i] * 7;
    }
    bb.ns_t.assign(b->ns_t, b->ns_t + n);
    bb.na_t.assign(b->na_t, b->na_t + n);
    bb.nm_t.assign(b->nm_t, b->nm_t + n);
    bb.nr_t.assign(b->nr_t, b->nr_t + n);
    bb.sect_t.assign(b->sect_t, b->sect_t + nt);
    bb.aoa_t.assign(b->aoa_t, b->aoa_t + na);
    bb.mach_t.assign(b->mach_t, b->mach_t + nm);
    bb.re_t.assign(b->re_t, b->re_t + nr);
    bb.table.assign(b->table, b->table + ntab);
    ctx->bb = std::move(bb);
    ctx->have_bb = true;
    ctx->bb_dirty = true;
    return ACUM_OK;
}

extern "C" int acum_bpm(acum_ctx* ctx, int aa_mode, double* BBspl, double* BBoaspl)
{
    acum::NvtxRange nvtx_range_("acum_bpm");
    if (!ctx) return ACUM_ERR_INVALID;
    ctx->begin_run();
    return bpm_run(ctx, aa_mode, nullptr, nullptr, BBspl, BBoaspl);
}

extern "C" int acum_find_bb_noise(int nSurf_BB, int nObs, int nTime, float dTau, const float* span, const float* omega,
                                  const int* ccw, const float* psi_offset, const int* trip, const float* rotate,
                                  const float* translate, const int* xsPtr, const int* dsPtr, const int* nsect,
                                  const float* xyzcR, const float* bbdata, const int* nsect_t, const int* nmach_t,
                                  const int* naoa_t, const int* nre_t, const int* aPtr, const int* mPtr,
                                  const int* rPtr, const int* sPtr, const int* dPtr, const float* sect_t,
                                  const float* mach_t, const float* aoa_t, const float* re_t, const float* bbdata_t,
                                  int t_del, const float* vInf, const float* rObs, const float* tObs, int nf2,
                                  const float* ff, float a0, float* BBspl, float* BBoaspl)
{
    acum::NvtxRange nvtx_range_("acum_find_bb_noise");
    (void)tObs;
    if (nSurf_BB <= 0 || nObs <= 0 || nTime < 6 || !span || !omega || !ccw || !psi_offset || !trip || !rotate ||
        !translate || !xsPtr || !dsPtr || !nsect || !xyzcR || !bbdata || !nsect_t || !nmach_t || !naoa_t || !nre_t ||
        !aPtr || !mPtr || !rPtr || !sPtr || !dPtr || !sect_t || !mach_t || !aoa_t || !re_t || !bbdata_t || !vInf ||
        !rObs || !ff || !BBspl || !BBoaspl)
        return fail(nullptr, ACUM_ERR_INVALID, "findBBnoise: bad argument");
    if (nf2 != kBands) return fail(nullptr, ACUM_ERR_UNSUPPORTED, "findBBnoise: the band table must have 42 bands");
    for (int i = 0; i < kBands; ++i)
        if (fabs((double)ff[i] - kBandHz[i]) > 1e-6 * kBandHz[i])
            return fail(nullptr, ACUM_ERR_UNSUPPORTED, "findBBnoise: the band table must be the 1/3-octave table");
    int dev = 0;
    cudaGetDevice(&dev);
    acum_ctx* c = nullptr;
    if (acum_create(&c, dev) != ACUM_OK) return fail(nullptr, ACUM_ERR_CUDA, "findBBnoise: cannot create a context");
    // a context holds the observers and the step size; the tonal surfaces are a dummy
    acum_inputs in;
    memset(&in, 0, sizeof(in));
    in.a0 = a0;
    in.rhoRef = 1.0;
    in.oM = 1.0;
    in.dPsi = 1.0;
    in.OBSscale = 1.0;
    in.CFDscale = 1.0;
    in.nTime = nTime;
    in.impermeable = 1;
    in.periodic = 1;
    std::vector<float> dummy((size_t)nTime * 8, 0.f);
    const int ns_dummy = std::max(1, nSurf_BB);
    std::vector<int> ne(ns_dummy, 1);
    std::vector<float> dummy_all((size_t)nTime * 8 * ns_dummy, 0.f);
    int rc = acum_set_deck(c, &in, nObs, rObs, ns_dummy, ne.data(), dummy_all.data(), 0);
    if (rc) {
        acum_destroy(c);
        return rc;
    }
    c->der.dTau = dTau;
    for (int i = 0; i < 3; ++i) c->der.vinf[i] = vInf[i];
    BBDeck bb;
    const int n = nSurf_BB;
    bb.nsurf = n;
    bb.t_del = t_del;
    for (int i = 0; i < n; ++i) {
        bb.span.push_back(span[i]);
        bb.omega.push_back(omega[i]);
        bb.psi_offset.push_back(psi_offset[i]);
        bb.ccw.push_back(ccw[i]);
        bb.trip.push_back(trip[i]);
        bb.nsect.push_back(nsect[i]);
        for (int k = 0; k < 3; ++k) {
            bb.rotate.push_back(rotate[3 * i + k]);
            bb.translate.push_back(translate[3 * i + k]);
        }
        for (int k = 0; k < 4 * nsect[i]; ++k) bb.geom.push_back(xyzcR[xsPtr[i] + k]);
        // bbdata arrives as read (cn, cc already divided)
        for (long long k = 0; k < (long long)nTime * nsect[i] * 7; ++k) bb.data.push_back(bbdata[dsPtr[i] + k]);
        bb.ns_t.push_back(nsect_t[i]);
        bb.na_t.push_back(naoa_t[i]);
        bb.nm_t.push_back(nmach_t[i]);
        bb.nr_t.push_back(nre_t[i]);
        for (int k = 0; k < nsect_t[i]; ++k) bb.sect_t.push_back(sect_t[sPtr[i] + k]);
        for (int k = 0; k < naoa_t[i]; ++k) bb.aoa_t.push_back(aoa_t[aPtr[i] + k]);
        for (int k = 0; k < nmach_t[i]; ++k) bb.mach_t.push_back(mach_t[mPtr[i] + k]);
        for (int k = 0; k < nre_t[i]; ++k) bb.re_t.push_back(re_t[rPtr[i] + k]);
        for (long long k = 0; k < (long long)nsect_t[i] * naoa_t[i] * nmach_t[i] * nre_t[i] * 7; ++k)
            bb.table.push_back(bbdata_t[dPtr[i] + k]);
    }
    c->bb = std::move(bb);
    c->have_bb = true;
    c->bb_dirty = true;
    std::vector<double> sspl((size_t)nObs * kBands * 7), soas(nObs), spl(sspl.size()), oas(nObs);
    for (size_t i = 0; i < sspl.size(); ++i) sspl[i] = BBspl[i];
    for (int i = 0; i < nObs; ++i) soas[i] = BBoaspl[i];
    rc = bpm_run(c, 0, sspl.data(), soas.data(), spl.data(), oas.data());
    if (rc == ACUM_OK) {
        for (size_t i = 0; i < spl.size(); ++i) BBspl[i] = (float)spl[i];
        for (int i = 0; i < nObs; ++i) BBoaspl[i] = (float)oas[i];
    }
    std::string msg = c->err;
    acum_destroy(c);
    if (rc) return fail(nullptr, rc, msg);
    return ACUM_OK;
}
