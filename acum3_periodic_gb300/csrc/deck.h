// deck.h -- host-side deck held by a context (the reference's global input state,
// variables.cuh, as one value), and the format readers/writers of io.cpp.
#pragma once

#include <string>
#include <vector>

#include "../../include/acum.h"

namespace acum {

// 1/3-octave band centres of the broadband model (io.cu:693-699)
constexpr int kBands = 42;
extern const double kBandHz[kBands];

struct BBDeck {
    int nsurf = 0, t_del = 0;
    std::vector<double> span, omega, psi_offset, rotate, translate;
    std::vector<int> ccw, trip, nsect;
    std::vector<double> geom;  // [sum nsect][4]
    std::vector<double> data;  // [surf][T][nsect][7], cn/cc divided by (r/R)^2 as read
    std::vector<int> ns_t, na_t, nm_t, nr_t;
    std::vector<double> sect_t, aoa_t, mach_t, re_t, table;  // table [s][m][r][a][7]
};

bool read_inputs(const std::string& dir, acum_inputs& in, int& nsurf, std::string* err);
bool read_observers(const std::string& dir, std::vector<float>& obs, int& nobs, std::string* err);
// surface rows of `ncol` floats: 8 (impermeable decks) or 12 (permeable decks)
inline int surface_columns(int impermeable) { return impermeable == 0 ? 12 : 8; }
bool read_surfaces(const std::string& dir, int nsurf, int ntime, int ncol, std::vector<int>& nelem,
                   std::vector<float>& raw, std::string* err);
bool write_surface_cache(const std::string& dir, int nsurf, int ntime, int ncol, const std::vector<int>& nelem,
                         const std::vector<float>& raw, std::string* err);
bool read_bb(const std::string& dir, int nsurf, int ntime, BBDeck& bb, std::string* err);
bool write_time_history(const std::string& dir, int T, int O, double dpsi_deg, const double* pT, const double* pL,
                        const double* pA, std::string* err);
bool write_bb_output(const std::string& dir, int O, const double* oaspl, const double* spl, const double* ff, int nf,
                     std::string* err);

}  // namespace acum
