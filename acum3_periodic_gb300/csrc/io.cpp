// io.cpp -- the reference's deck formats (io.cu) on the host: readers for input,
// obs.dat, surfaces/surface_<i>.dat, input_BB, BB_inputs/BB_surface_<i>.dat and
// BB_inputs/BB_table_<i>.dat, and writers for pT.out, pL.out, pA.out, bb_oaspl.out and
// bb_spl.dat.  Numbers are parsed with strtod (correctly rounded, like fscanf); surface
// rows are stored as float, as read_surf stores them.  Large surface files are parsed in
// parallel over line-aligned chunks.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <sys/stat.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <thread>
#include <vector>

#include "deck.h"

namespace acum {

static bool slurp(const std::string& path, std::string& out)
{
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return false;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    out.resize(n > 0 ? (size_t)n : 0);
    size_t got = n > 0 ? fread(&out[0], 1, (size_t)n, f) : 0;
    fclose(f);
    out.resize(got);
    return true;
}

static std::vector<std::string> tokens(const std::string& s)
{
    std::vector<std::string> t;
    size_t i = 0, n = s.size();
    while (i < n) {
        while (i < n && isspace((unsigned char)s[i])) ++i;
        size_t j = i;
        while (j < n && !isspace((unsigned char)s[j])) ++j;
        if (j > i) t.emplace_back(s.substr(i, j - i));
        i = j;
    }
    return t;
}

// parses whitespace-separated reals from [p, end) into out (up to `want` values)
static size_t parse_reals(const char* p, const char* end, float* out, size_t want)
{
    size_t k = 0;
    while (k < want) {
        while (p < end && isspace((unsigned char)*p)) ++p;
        if (p >= end) break;
        char* q;
        double v = strtod(p, &q);
        if (q == p) break;
        out[k++] = (float)v;
        p = q;
    }
    return k;
}

static size_t parse_reals_d(const char* p, const char* end, double* out, size_t want, const char** stop)
{
    size_t k = 0;
    while (k < want) {
        while (p < end && isspace((unsigned char)*p)) ++p;
        if (p >= end) break;
        char* q;
        double v = strtod(p, &q);
        if (q == p) break;
        out[k++] = v;
        p = q;
    }
    if (stop) *stop = p;
    return k;
}

// Parses `count` rows of `ncol` reals starting at `p`, with several threads over
// line-aligned slices.  Returns false if the text holds fewer numbers.
static bool parse_rows_parallel(const char* p, const char* end, int ncol, size_t count, float* out)
{
    const size_t want = count * (size_t)ncol;
    const size_t bytes = (size_t)(end - p);
    int nth = (int)std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()), 32);
    if (bytes < (8u << 20)) nth = 1;
    // slice at line starts, then count the rows of each slice
    std::vector<const char*> cut(nth + 1);
    cut[0] = p;
    cut[nth] = end;
    for (int i = 1; i < nth; ++i) {
        const char* c = p + bytes * i / nth;
        while (c < end && *c != '\n') ++c;
        cut[i] = c < end ? c + 1 : end;
    }
    std::vector<size_t> rows(nth, 0);
    auto count_lines = [&](int i) {
        size_t r = 0;
        const char* c = cut[i];
        while (c < cut[i + 1]) {
            const char* s = c;
            while (c < cut[i + 1] && *c != '\n') ++c;
            bool blank = true;
            for (const char* x = s; x < c; ++x)
                if (!isspace((unsigned char)*x)) { blank = false; break; }
            if (!blank) ++r;
            if (c < cut[i + 1]) ++c;
        }
        rows[i] = r;
    };
    {
        std::vector<std::thread> th;
        for (int i = 1; i < nth; ++i) th.emplace_back(count_lines, i);
        count_lines(0);
        for (auto& t : th) t.join();
    }
    std::vector<size_t> start(nth, 0);
    for (int i = 1; i < nth; ++i) start[i] = start[i - 1] + rows[i - 1];
    std::vector<size_t> got(nth, 0);
    auto work = [&](int i) {
        if (start[i] >= count) return;
        size_t rmax = std::min(rows[i], count - start[i]);
        got[i] = parse_reals(cut[i], cut[i + 1], out + start[i] * ncol, rmax * ncol);
    };
    {
        std::vector<std::thread> th;
        for (int i = 1; i < nth; ++i) th.emplace_back(work, i);
        work(0);
        for (auto& t : th) t.join();
    }
    size_t tot = 0;
    for (int i = 0; i < nth; ++i) tot += got[i];
    return tot >= want;
}

static bool set_err(std::string* err, const std::string& m)
{
    if (err) *err = m;
    return false;
}

// io.cu:12-101
bool read_inputs(const std::string& dir, acum_inputs& in, int& nsurf, std::string* err)
{
    std::string s;
    if (!slurp(dir + "/input", s)) return set_err(err, "No input file found in " + dir);
    in.a0 = 340.0;
    in.rhoRef = 1.2;
    in.pRef = 0.0;
    in.nTime = 360;
    in.dPsi = 1.0;
    in.xy_angle = 0.0;
    in.xz_angle = 0.0;
    in.periodic = 1;
    in.lowpass = 1;
    in.BB_noise = 0;
    in.Mref = 0.08;
    in.impermeable = 0;
    in.oM = 0.0;
    in.Minf = 0.0;
    in.CFDscale = 0.0;
    in.OBSscale = 0.0;
    nsurf = 0;
    std::vector<std::string> t = tokens(s);
    for (size_t i = 0; i < t.size(); ++i) {
        const std::string& k = t[i];
        auto num = [&](double& v) -> bool {
            if (i + 1 >= t.size()) return false;
            v = (float)strtod(t[++i].c_str(), nullptr);  // the reference reads these as float
            return true;
        };
        auto inum = [&](int& v) -> bool {
            if (i + 1 >= t.size()) return false;
            v = atoi(t[++i].c_str());
            return true;
        };
        bool ok = true;
        if (k == "a0") ok = num(in.a0);
        else if (k == "impermeable") ok = inum(in.impermeable);
        else if (k == "rhoRef") ok = num(in.rhoRef);
        else if (k == "pRef") ok = num(in.pRef);
        else if (k == "oM") ok = num(in.oM);
        else if (k == "nSurf") ok = inum(nsurf);
        else if (k == "nTime") ok = inum(in.nTime);
        else if (k == "dPsi") ok = num(in.dPsi);
        else if (k == "Minf") ok = num(in.Minf);
        else if (k == "Mref") ok = num(in.Mref);
        else if (k == "xy_angle") ok = num(in.xy_angle);
        else if (k == "xz_angle") ok = num(in.xz_angle);
        else if (k == "CFDscale") ok = num(in.CFDscale);
        else if (k == "OBSscale") ok = num(in.OBSscale);
        else if (k == "periodic") ok = inum(in.periodic);
        else if (k == "lowpass") ok = inum(in.lowpass);
        else if (k == "BB_noise") ok = inum(in.BB_noise);
        else if (k == "ACUM-3_INPUTS" || k == "***Environmental" || k == "***Geometric" || k == "***Data") continue;
        else return set_err(err, "Input parameter not defined: " + k);
        if (!ok) return set_err(err, "Missing value for input parameter " + k);
    }
    return true;
}

// io.cu:106-135
bool read_observers(const std::string& dir, std::vector<float>& obs, int& nobs, std::string* err)
{
    std::string s;
    if (!slurp(dir + "/obs.dat", s)) return set_err(err, "Unable to open observer file: obs.dat");
    const char* p = s.c_str();
    char* q;
    long n = strtol(p, &q, 10);
    if (q == p || n < 0) return set_err(err, "obs.dat: bad observer count");
    nobs = (int)n;
    obs.assign((size_t)nobs * 3, 0.f);
    size_t got = parse_reals(q, s.c_str() + s.size(), obs.data(), obs.size());
    if (got < obs.size()) return set_err(err, "obs.dat: fewer coordinates than observers");
    return true;
}

// Binary cache of the surface rows (surfaces/surfaces.acumbin): the float rows exactly as
// read from the text files (8 columns per row for impermeable decks, 12 for permeable
// ones), with the size and modification time of each text file, so a later load skips
// the text parse when none of them changed.
namespace {
const char kCacheMagic[8] = {'A', 'C', 'U', 'M', 'S', 'R', 'F', '2'};

struct FileStamp {
    int64_t size, mtime_ns;
};

bool stamp_of(const std::string& fn, FileStamp& st)
{
    struct stat sb;
    if (stat(fn.c_str(), &sb) != 0) return false;
    st.size = (int64_t)sb.st_size;
    st.mtime_ns = (int64_t)sb.st_mtim.tv_sec * 1000000000LL + (int64_t)sb.st_mtim.tv_nsec;
    return true;
}

std::string surface_file(const std::string& dir, int i)
{
    return dir + "/surfaces/surface_" + std::to_string(i + 1) + ".dat";
}

std::string cache_file(const std::string& dir) { return dir + "/surfaces/surfaces.acumbin"; }

// rows from the cache if it exists and matches every text file and the row width; false
// otherwise
bool read_surface_cache(const std::string& dir, int nsurf, int ntime, int ncol, std::vector<int>& nelem,
                        std::vector<float>& raw)
{
    FILE* f = fopen(cache_file(dir).c_str(), "rb");
    if (!f) return false;
    bool ok = false;
    char magic[8];
    int32_t ns = 0, nt = 0, nc = 0;
    if (fread(magic, 1, 8, f) == 8 && memcmp(magic, kCacheMagic, 8) == 0 && fread(&ns, 4, 1, f) == 1 &&
        fread(&nt, 4, 1, f) == 1 && fread(&nc, 4, 1, f) == 1 && ns == nsurf && nt == ntime && nc == ncol) {
        std::vector<int32_t> ne(ns);
        std::vector<FileStamp> st(ns);
        ok = fread(ne.data(), 4, ns, f) == (size_t)ns && fread(st.data(), sizeof(FileStamp), ns, f) == (size_t)ns;
        size_t total = 0;
        for (int i = 0; ok && i < ns; ++i) {
            FileStamp now;
            ok = ne[i] >= 0 && stamp_of(surface_file(dir, i), now) && now.size == st[i].size &&
                 now.mtime_ns == st[i].mtime_ns;
            total += (size_t)ntime * ne[i] * ncol;
        }
        if (ok) {
            raw.assign(total, 0.f);
            ok = fread(raw.data(), 4, total, f) == total;
            if (ok) nelem.assign(ne.begin(), ne.end());
        }
    }
    fclose(f);
    if (!ok) raw.clear();
    return ok;
}
}  // namespace

bool write_surface_cache(const std::string& dir, int nsurf, int ntime, int ncol, const std::vector<int>& nelem,
                         const std::vector<float>& raw, std::string* err)
{
    std::vector<FileStamp> st(nsurf);
    for (int i = 0; i < nsurf; ++i)
        if (!stamp_of(surface_file(dir, i), st[i])) return set_err(err, "Unable to stat " + surface_file(dir, i));
    const std::string tmp = cache_file(dir) + ".tmp";
    FILE* f = fopen(tmp.c_str(), "wb");
    if (!f) return set_err(err, "Unable to write " + tmp);
    const int32_t ns = nsurf, nt = ntime, nc = ncol;
    std::vector<int32_t> ne(nelem.begin(), nelem.end());
    bool ok = fwrite(kCacheMagic, 1, 8, f) == 8 && fwrite(&ns, 4, 1, f) == 1 && fwrite(&nt, 4, 1, f) == 1 &&
              fwrite(&nc, 4, 1, f) == 1 && fwrite(ne.data(), 4, ns, f) == (size_t)ns &&
              fwrite(st.data(), sizeof(FileStamp), ns, f) == (size_t)ns &&
              fwrite(raw.data(), 4, raw.size(), f) == raw.size();
    ok = (fclose(f) == 0) && ok;
    if (!ok || rename(tmp.c_str(), cache_file(dir).c_str()) != 0) {
        remove(tmp.c_str());
        return set_err(err, "Unable to write " + cache_file(dir));
    }
    return true;
}

// io.cu:206-333: rows of 8 columns x y z Cp A nx ny nz for impermeable decks (io.cu:321),
// of 12 columns x y z u v w P rho ds nx ny nz for permeable ones (io.cu:286)
bool read_surfaces(const std::string& dir, int nsurf, int ntime, int ncol, std::vector<int>& nelem,
                   std::vector<float>& raw, std::string* err)
{
    if (ncol != 8 && ncol != 12) return set_err(err, "surface rows have 8 or 12 columns");
    if (read_surface_cache(dir, nsurf, ntime, ncol, nelem, raw)) return true;
    nelem.assign(nsurf, 0);
    std::vector<std::string> bufs(nsurf);
    size_t total = 0;
    for (int i = 0; i < nsurf; ++i) {
        std::string fn = dir + "/surfaces/surface_" + std::to_string(i + 1) + ".dat";
        if (!slurp(fn, bufs[i])) return set_err(err, "Unable to open surface file " + fn);
        int e = 0, nt = 0;
        if (sscanf(bufs[i].c_str(), "%d %d", &e, &nt) != 2 || e < 0)
            return set_err(err, "Bad header in " + fn);
        if (nt != ntime) {
            // the reference prints "Inconsistent number of steps" and carries on with
            // nTime rows per element; so does this reader
        }
        nelem[i] = e;
        total += (size_t)ntime * e * ncol;
    }
    raw.assign(total, 0.f);
    size_t off = 0;
    for (int i = 0; i < nsurf; ++i) {
        const char* p = bufs[i].c_str();
        const char* end = p + bufs[i].size();
        while (p < end && *p != '\n') ++p;  // header line
        const size_t rows = (size_t)ntime * nelem[i];
        if (!parse_rows_parallel(p, end, ncol, rows, raw.data() + off))
            return set_err(err, "surfaces/surface_" + std::to_string(i + 1) + ".dat: fewer rows than nTime*E");
        off += rows * ncol;
        std::string().swap(bufs[i]);
    }
    return true;
}

// io.cu:337-700
bool read_bb(const std::string& dir, int nsurf, int ntime, BBDeck& bb, std::string* err)
{
    std::string s;
    if (!slurp(dir + "/input_BB", s)) return set_err(err, "No broadband input file found");
    std::vector<std::string> t = tokens(s);
    int nbb = nsurf;
    bb.t_del = 0;
    auto resize = [&](int n) {
        bb.nsurf = n;
        bb.span.assign(n, 1.0);
        bb.omega.assign(n, 1.0);
        bb.ccw.assign(n, 1);
        bb.psi_offset.assign(n, 0.0);
        bb.trip.assign(n, 0);
        bb.rotate.assign(3 * n, 0.0);
        bb.translate.assign(3 * n, 0.0);
    };
    resize(nbb);
    int cur = 0;
    for (size_t i = 0; i < t.size(); ++i) {
        const std::string& k = t[i];
        auto num = [&]() -> double { return i + 1 < t.size() ? (float)strtod(t[++i].c_str(), nullptr) : 0.0; };
        if (k == "ACUM-3_Broadband_Inputs" || k == "Initial_Position") continue;
        if (k == "nSurf_BB") {
            nbb = i + 1 < t.size() ? atoi(t[++i].c_str()) : 0;
            if (nbb > nsurf)
                return set_err(err, "Number of surfaces considered for broadband noise cannot be higher than the "
                                    "available surfaces");
            resize(nbb);
        } else if (k == "t_del") {
            bb.t_del = i + 1 < t.size() ? atoi(t[++i].c_str()) : 0;
        } else if (k == "***Surface-" + std::to_string(cur + 1)) {
            cur += 1;
        } else if (cur < 1 || cur > nbb) {
            return set_err(err, "Input parameter not defined: " + k);
        } else if (k == "span(m)") bb.span[cur - 1] = num();
        else if (k == "omega(rad/s)") bb.omega[cur - 1] = num();
        else if (k == "ccw") bb.ccw[cur - 1] = i + 1 < t.size() ? atoi(t[++i].c_str()) : 1;
        else if (k == "psi_offset") bb.psi_offset[cur - 1] = num();
        else if (k == "trip") bb.trip[cur - 1] = i + 1 < t.size() ? atoi(t[++i].c_str()) : 0;
        else if (k == "rotate") {
            for (int c = 0; c < 3; ++c) bb.rotate[3 * (cur - 1) + c] = num();
        } else if (k == "translate") {
            for (int c = 0; c < 3; ++c) bb.translate[3 * (cur - 1) + c] = num();
            if (cur == nbb) break;
        } else {
            return set_err(err, "Input parameter not defined: " + k);
        }
    }
    bb.nsect.assign(nbb, 0);
    bb.geom.clear();
    bb.data.clear();
    for (int i = 0; i < nbb; ++i) {
        std::string fn = dir + "/BB_inputs/BB_surface_" + std::to_string(i + 1) + ".dat";
        std::string b;
        if (!slurp(fn, b)) return set_err(err, "Unable to open " + fn);
        int nt = 0, ns = 0;
        if (sscanf(b.c_str(), "%d %d", &nt, &ns) != 2 || ns < 3) return set_err(err, "Bad header in " + fn);
        bb.nsect[i] = ns;
        const char* p = b.c_str();
        const char* end = p + b.size();
        while (p < end && *p != '\n') ++p;
        std::vector<double> g((size_t)ns * 4), d((size_t)ntime * ns * 7);
        const char* stop = p;
        if (parse_reals_d(p, end, g.data(), g.size(), &stop) < g.size()) return set_err(err, fn + ": short");
        if (parse_reals_d(stop, end, d.data(), d.size(), nullptr) < d.size()) return set_err(err, fn + ": short");
        // float storage as read (fscanf %e into float), then cn, cc divided by (r/R)^2
        for (auto& v : g) v = (double)(float)v;
        for (auto& v : d) v = (double)(float)v;
        if ((float)bb.omega[i] != 0.0f) {
            for (int tt = 0; tt < ntime; ++tt)
                for (int k = 0; k < ns; ++k) {
                    double rr = g[4 * k];
                    d[((size_t)tt * ns + k) * 7 + 4] /= rr * rr;
                    d[((size_t)tt * ns + k) * 7 + 5] /= rr * rr;
                }
        }
        bb.geom.insert(bb.geom.end(), g.begin(), g.end());
        bb.data.insert(bb.data.end(), d.begin(), d.end());
    }
    bb.ns_t.assign(nbb, 0);
    bb.na_t.assign(nbb, 0);
    bb.nm_t.assign(nbb, 0);
    bb.nr_t.assign(nbb, 0);
    bb.sect_t.clear();
    bb.aoa_t.clear();
    bb.mach_t.clear();
    bb.re_t.clear();
    bb.table.clear();
    for (int i = 0; i < nbb; ++i) {
        std::string fn = dir + "/BB_inputs/BB_table_" + std::to_string(i + 1) + ".dat";
        std::string b;
        if (!slurp(fn, b)) return set_err(err, "Unable to open " + fn);
        const char* p = b.c_str();
        const char* end = p + b.size();
        while (p < end && *p != '\n') ++p;  // VARIABLES= line
        int ns, na, nm, nr;
        if (sscanf(p, "%d %d %d %d", &ns, &na, &nm, &nr) != 4 || ns < 1 || na < 2 || nm < 1 || nr < 1)
            return set_err(err, "Bad header in " + fn);
        ++p;
        while (p < end && *p != '\n') ++p;
        bb.ns_t[i] = ns;
        bb.na_t[i] = na;
        bb.nm_t[i] = nm;
        bb.nr_t[i] = nr;
        std::vector<double> sect(ns), aoa(na), mach(nm), re(nr), tab((size_t)ns * nm * nr * na * 7);
        const char* q = p;
        for (int j = 0; j < ns; ++j) {
            double v;
            if (parse_reals_d(q, end, &v, 1, &q) < 1) return set_err(err, fn + ": short");
            sect[j] = (float)v;
            std::vector<double> row(10);
            for (int k = 0; k < nm; ++k)
                for (int l = 0; l < nr; ++l)
                    for (int m = 0; m < na; ++m) {
                        if (parse_reals_d(q, end, row.data(), 10, &q) < 10) return set_err(err, fn + ": short");
                        aoa[m] = (float)row[0];
                        mach[k] = (float)row[1];
                        for (int c = 0; c < 7; ++c)
                            tab[((((size_t)j * nm + k) * nr + l) * na + m) * 7 + c] = (float)row[2 + c];
                        re[l] = (float)row[9];
                    }
        }
        // table validation of io.cu:628-687
        for (int j = 0; j < ns; ++j) {
            if (sect[j] < 0.0 || sect[j] > 1.0) return set_err(err, "Check span section of " + fn);
            for (int k = 0; k < ns; ++k)
                if (j != k && sect[j] == sect[k]) return set_err(err, "Check span sections of " + fn);
        }
        for (int j = 0; j < nm; ++j) {
            if (mach[j] < 0.0) return set_err(err, "Check Mach numbers of " + fn);
            for (int k = 0; k < nm; ++k)
                if (j != k && mach[j] == mach[k]) return set_err(err, "Check Mach numbers of " + fn);
        }
        for (int j = 0; j < nr; ++j) {
            if (re[j] < 0.0) return set_err(err, "Check Re numbers of " + fn);
            for (int k = 0; k < nr; ++k)
                if (j != k && re[j] == re[k]) return set_err(err, "Check Re numbers of " + fn);
        }
        for (int j = 0; j < na; ++j)
            for (int k = 0; k < na; ++k)
                if (j != k && aoa[j] == aoa[k]) return set_err(err, "Check AoAs of " + fn);
        bb.sect_t.insert(bb.sect_t.end(), sect.begin(), sect.end());
        bb.aoa_t.insert(bb.aoa_t.end(), aoa.begin(), aoa.end());
        bb.mach_t.insert(bb.mach_t.end(), mach.begin(), mach.end());
        bb.re_t.insert(bb.re_t.end(), re.begin(), re.end());
        bb.table.insert(bb.table.end(), tab.begin(), tab.end());
    }
    return true;
}

// io.cu:137-203
bool write_time_history(const std::string& dir, int T, int O, double dpsi_deg, const double* pT, const double* pL,
                        const double* pA, std::string* err)
{
    const float dpsi = (float)(dpsi_deg * M_PI / 180.0);
    const char* names[3] = {"pT.out", "pL.out", "pA.out"};
    const double* arr[3] = {pT, pL, pA};
    for (int k = 0; k < 3; ++k) {
        std::string fn = dir + "/" + names[k];
        FILE* f = fopen(fn.c_str(), "w");
        if (!f) return set_err(err, "cannot write " + fn);
        fprintf(f, "# ntime nobs\n");
        fprintf(f, "%d %d\n", T, O);
        for (int i = 0; i < T; ++i) {
            fprintf(f, " %14.8E", (double)((float)i * dpsi));
            for (int j = 0; j < O; ++j) fprintf(f, " %14.8E", arr[k][(size_t)i * O + j]);
            fprintf(f, "\n");
        }
        fclose(f);
    }
    return true;
}

// io.cu:702-796
bool write_bb_output(const std::string& dir, int O, const double* oaspl, const double* spl, const double* ff, int nf,
                     std::string* err)
{
    std::string fn = dir + "/bb_oaspl.out";
    FILE* f = fopen(fn.c_str(), "w");
    if (!f) return set_err(err, "cannot write " + fn);
    fprintf(f, "nobs: %d\n", O);
    for (int i = 0; i < O; ++i) fprintf(f, " %14.8E\n", oaspl[i]);
    fclose(f);
    fn = dir + "/bb_spl.dat";
    f = fopen(fn.c_str(), "w");
    if (!f) return set_err(err, "cannot write " + fn);
    fprintf(f, " # nfrequency nobs\n    %d      %d\n", nf, O);
    static const char* zone[7] = {"TOTAL", "TBL_TE_P", "TBL_TE_S", "TBL_SS", "TEB_VS", "LBL-VS", "TVF"};
    static const int comp[7] = {0, 3, 2, 1, 5, 4, 6};
    for (int z = 0; z < 7; ++z) {
        fprintf(f, " ZONE T=\"%s\"\n", zone[z]);
        for (int j = 0; j < nf; ++j) {
            fprintf(f, "   %e", (double)(float)ff[j]);
            for (int i = 0; i < O; ++i) fprintf(f, "  %e", spl[((size_t)i * nf + j) * 7 + comp[z]]);
            fprintf(f, "\n");
        }
    }
    fclose(f);
    return true;
}

}  // namespace acum
