// ref_stubs.cxx -- definitions the reference's hot-path objects need at link
// time (TEST INFRASTRUCTURE ONLY; see ref_harness.h).  Nothing here changes
// the arithmetic of the reference classes that are compiled unchanged; the
// restated parts (grid metrics, thermodynamics, ghost cells) follow the cited
// reference lines.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "ref_harness.h"

#include "advec.h"
#include "diff.h"
#include "pres.h"
#include "fft.h"
#include "stats.h"
#include "column.h"
#include "cross.h"
#include "constants.h"
#include "field3d_io.h"
#include "cuda_buffer.h"
#include "netcdf_interface.h"

#include "../orc_fft.h"

using TF = double;

// ---------------------------------------------------------------------------
// Input: "group key subkey value" lines (subkey "-" for none).
// ---------------------------------------------------------------------------
Input::Input(Master& masterin, const std::string& text) : master(masterin)
{
    std::istringstream ss(text);
    std::string line;
    while (std::getline(ss, line))
    {
        std::istringstream ls(line);
        std::string g, k, s, v;
        if (!(ls >> g >> k >> s)) continue;
        std::getline(ls, v);
        v.erase(0, v.find_first_not_of(" \t"));
        if (s == "-") s = "";
        itemlist[g][k][s] = std::make_pair(v, false);
    }
}

namespace
{
    template<typename T> T parse_item(const std::string& v);
    template<> int parse_item<int>(const std::string& v) { return std::stoi(v); }
    template<> double parse_item<double>(const std::string& v) { return std::stod(v); }
    template<> float parse_item<float>(const std::string& v) { return std::stof(v); }
    template<> std::string parse_item<std::string>(const std::string& v) { return v; }
    template<> bool parse_item<bool>(const std::string& v)
    {
        if (v == "1" || v == "true") return true;
        if (v == "0" || v == "false") return false;
        throw std::runtime_error("bad bool item " + v);
    }
}

template<typename T>
T Input::get_item(const std::string& g, const std::string& k, const std::string& s)
{
    auto it = itemlist.find(g);
    if (it != itemlist.end())
    {
        auto it2 = it->second.find(k);
        if (it2 != it->second.end())
        {
            auto it3 = it2->second.find(s);
            if (it3 == it2->second.end()) it3 = it2->second.find("");
            if (it3 != it2->second.end())
                return parse_item<T>(it3->second.first);
        }
    }
    throw std::runtime_error("missing input item " + g + "." + k + "[" + s + "]");
}

template<typename T>
T Input::get_item(const std::string& g, const std::string& k, const std::string& s, const T def)
{
    try { return get_item<T>(g, k, s); }
    catch (std::runtime_error&) { return def; }
}

template<typename T>
std::vector<T> Input::get_list(const std::string& g, const std::string& k, const std::string& s)
{
    std::string v = get_item<std::string>(g, k, s);
    std::vector<T> out;
    std::stringstream ss(v);
    std::string tok;
    while (std::getline(ss, tok, ','))
    {
        tok.erase(0, tok.find_first_not_of(" \t"));
        if (!tok.empty()) out.push_back(parse_item<T>(tok));
    }
    return out;
}

template<typename T>
std::vector<T> Input::get_list(const std::string& g, const std::string& k, const std::string& s, const std::vector<T> def)
{
    try { return get_list<T>(g, k, s); }
    catch (std::runtime_error&) { return def; }
}

void Input::flag_as_used(const std::string&, const std::string&, const std::string&) {}
void Input::print_unused_items() {}

template int Input::get_item<int>(const std::string&, const std::string&, const std::string&);
template double Input::get_item<double>(const std::string&, const std::string&, const std::string&);
template bool Input::get_item<bool>(const std::string&, const std::string&, const std::string&);
template std::string Input::get_item<std::string>(const std::string&, const std::string&, const std::string&);
template int Input::get_item<int>(const std::string&, const std::string&, const std::string&, const int);
template double Input::get_item<double>(const std::string&, const std::string&, const std::string&, const double);
template bool Input::get_item<bool>(const std::string&, const std::string&, const std::string&, const bool);
template std::string Input::get_item<std::string>(const std::string&, const std::string&, const std::string&, const std::string);
template std::vector<std::string> Input::get_list<std::string>(const std::string&, const std::string&, const std::string&);
template std::vector<std::string> Input::get_list<std::string>(const std::string&, const std::string&, const std::string&, const std::vector<std::string>);

// ---------------------------------------------------------------------------
// cuda_raw_buffer: the CPU build never allocates device memory.
// ---------------------------------------------------------------------------
cuda_raw_buffer::cuda_raw_buffer(size_t n) { if (n) throw std::runtime_error("no device memory in the CPU harness"); }
cuda_raw_buffer::cuda_raw_buffer(cuda_raw_buffer&& that) noexcept { ptr_ = that.ptr_; that.ptr_ = nullptr; }
cuda_raw_buffer& cuda_raw_buffer::operator=(cuda_raw_buffer&& that) noexcept { std::swap(ptr_, that.ptr_); return *this; }
void cuda_raw_buffer::reallocate(size_t n) { if (n) throw std::runtime_error("no device memory in the CPU harness"); }

// ---------------------------------------------------------------------------
// Transpose (serial: never called on the hot path)
// ---------------------------------------------------------------------------
template<typename T> Transpose<T>::Transpose(Master& m, Grid<T>& g) : master(m), grid(g) { mpi_types_allocated = false; }
template<typename T> Transpose<T>::~Transpose() {}
template<typename T> void Transpose<T>::init() {}
template class Transpose<double>;

// ---------------------------------------------------------------------------
// Grid: constructor after src/grid.cxx:47-100, init after :105-193,
// 2nd-order metrics after :245-305.
// ---------------------------------------------------------------------------
namespace { std::vector<double> pending_z; }
void ref_harness::set_pending_z(const std::vector<double>& z) { pending_z = z; }

template<>
Grid<TF>::Grid(Master& masterin, Input& input) : master(masterin), transpose(master, *this)
{
    mpitypes = false;
    gd.xsize = input.get_item<TF>("grid", "xsize", "");
    gd.ysize = input.get_item<TF>("grid", "ysize", "");
    gd.zsize = input.get_item<TF>("grid", "zsize", "");
    gd.itot = input.get_item<int>("grid", "itot", "");
    gd.jtot = input.get_item<int>("grid", "jtot", "");
    gd.ktot = input.get_item<int>("grid", "ktot", "");
    gd.utrans = 0.; gd.vtrans = 0.;
    gd.lat = -9999.; gd.lon = -9999.;
    spatial_order = Grid_order::Second;
    gd.igc = 1; gd.jgc = 1; gd.kgc = 1;
    swtimedep = false;
}

template<> Grid<TF>::~Grid() {}

template<>
void Grid<TF>::set_minimum_ghost_cells(const int igcin, const int jgcin, const int kgcin)
{
    gd.igc = std::max(gd.igc, igcin);
    gd.jgc = std::max(gd.jgc, jgcin);
    gd.kgc = std::max(gd.kgc, kgcin);
}

template<> const Grid_data<TF>& Grid<TF>::get_grid_data() const { return gd; }

template<>
void Grid<TF>::init()
{
    gd.ntot = gd.itot*gd.jtot*gd.ktot;
    gd.imax = gd.itot; gd.jmax = gd.jtot; gd.kmax = gd.ktot;
    gd.nmax = gd.imax*gd.jmax*gd.kmax;
    gd.iblock = gd.itot; gd.jblock = gd.jtot; gd.kblock = gd.ktot;
    gd.icells = gd.imax + 2*gd.igc;
    gd.jcells = gd.jmax + 2*gd.jgc;
    gd.ijcells = gd.icells*gd.jcells;
    gd.kcells = gd.kmax + 2*gd.kgc;
    gd.ncells = gd.ijcells*gd.kcells;
    gd.istart = gd.igc; gd.jstart = gd.jgc; gd.kstart = gd.kgc;
    gd.iend = gd.imax + gd.igc; gd.jend = gd.jmax + gd.jgc; gd.kend = gd.kmax + gd.kgc;
    gd.istride = 1; gd.jstride = gd.icells; gd.kstride = gd.ijcells;
    gd.x.resize(gd.icells); gd.xh.resize(gd.icells);
    gd.y.resize(gd.jcells); gd.yh.resize(gd.jcells);
    for (auto* v : {&gd.z, &gd.zh, &gd.dz, &gd.dzh, &gd.dzi, &gd.dzhi, &gd.dzi4, &gd.dzhi4})
        v->assign(gd.kcells, 0.);
}

template<>
void Grid<TF>::calculate()
{
    gd.dx = gd.xsize / gd.itot;
    gd.dy = gd.ysize / gd.jtot;
    gd.dxi = 1./gd.dx;
    gd.dyi = 1./gd.dy;
    for (int i=0; i<gd.icells; ++i)
    {
        gd.x [i] = 0.5*gd.dx + (i-gd.igc)*gd.dx;
        gd.xh[i] = (i-gd.igc)*gd.dx;
    }
    for (int j=0; j<gd.jcells; ++j)
    {
        gd.y [j] = 0.5*gd.dy + (j-gd.jgc)*gd.dy;
        gd.yh[j] = (j-gd.jgc)*gd.dy;
    }
    gd.z[gd.kstart-1] = -gd.z[gd.kstart];
    gd.z[gd.kend]     = 2.*gd.zsize - gd.z[gd.kend-1];
    for (int k=gd.kstart+1; k<gd.kend; ++k)
        gd.zh[k] = 0.5*(gd.z[k-1]+gd.z[k]);
    gd.zh[gd.kstart] = 0.;
    gd.zh[gd.kend]   = gd.zsize;
    for (int k=1; k<gd.kcells; ++k)
    {
        gd.dzh [k] = gd.z[k] - gd.z[k-1];
        gd.dzhi[k] = 1./gd.dzh[k];
    }
    gd.dzh [gd.kstart-1] = gd.dzh [gd.kstart+1];
    gd.dzhi[gd.kstart-1] = gd.dzhi[gd.kstart+1];
    for (int k=1; k<gd.kcells-1; ++k)
    {
        gd.dz [k] = gd.zh[k+1] - gd.zh[k];
        gd.dzi[k] = 1./gd.dz[k];
    }
    gd.dz [gd.kstart-1] = gd.dz [gd.kstart];
    gd.dzi[gd.kstart-1] = gd.dzi[gd.kstart];
    gd.dz [gd.kend]     = gd.dz [gd.kend-1];
    gd.dzi[gd.kend]     = gd.dzi[gd.kend-1];
}

// The harness has no NetCDF: the z levels come from set_pending_z.
template<>
void Grid<TF>::create(Input&, Netcdf_handle&)
{
    for (int k=0; k<gd.ktot; ++k)
        gd.z[k + gd.kstart] = pending_z.at(k);
    calculate();
}

template class Grid<double>;

// ---------------------------------------------------------------------------
// Soil grid (disabled)
// ---------------------------------------------------------------------------
namespace { Soil_grid_data<TF> empty_soil_grid; }
template<> Soil_grid<TF>::Soil_grid(Master& m, Grid<TF>& g, Input&) : master(m), grid(g)
{
    empty_soil_grid.is_enabled = false;
    empty_soil_grid.kstart = 0; empty_soil_grid.kend = 0; empty_soil_grid.ncells = 0;
}
template<> Soil_grid<TF>::~Soil_grid() {}
template<> const Soil_grid_data<TF>& Soil_grid<TF>::get_grid_data() { return empty_soil_grid; }

// ---------------------------------------------------------------------------
// Fields: storage only; ref_driver.cxx registers u, v, w, th, p, evisc.
// ---------------------------------------------------------------------------
template<>
Fields<TF>::Fields(Master& m, Grid<TF>& g, Soil_grid<TF>& sg, Input& input) :
    master(m), grid(g), soil_grid(sg),
    field3d_io(master, grid), field3d_operators(master, grid, *this), boundary_cyclic(master, grid)
{
    calc_mean_profs = false;
    n_tmp_fields = 0;
    n_tmp_fields_xy = 0;
    visc = input.get_item<TF>("fields", "visc", "");
}

template<> Fields<TF>::~Fields() {}

template<>
void Fields<TF>::init_momentum_field(const std::string& name, const std::string& longname,
        const std::string& unit, const std::string& group, const std::array<int,3>& loc)
{
    mp[name] = std::make_shared<Field3d<TF>>(master, grid, name, longname, unit, group, loc);
    mt[name] = std::make_shared<Field3d<TF>>(master, grid, name + "t", longname, unit, group, loc);
    ap[name] = mp[name]; at[name] = mt[name];
    a[name] = mp[name];
    mp[name]->init(); mt[name]->init();
    mp[name]->visc = visc;
}

// src/fields.cxx:843-846 (only called with swupdate, which the path does not use)
template<>
void Fields<TF>::set_calc_mean_profs(bool sw) { calc_mean_profs = sw; }

template<>
void Fields<TF>::init_prognostic_field(const std::string& name, const std::string& longname,
        const std::string& unit, const std::string& group, const std::array<int,3>& loc, const bool& required)
{
    required_read[name] = required;   // src/fields.cxx:904
    sp[name] = std::make_shared<Field3d<TF>>(master, grid, name, longname, unit, group, loc);
    st[name] = std::make_shared<Field3d<TF>>(master, grid, name + "t", longname, unit, group, loc);
    ap[name] = sp[name]; at[name] = st[name];
    a[name] = sp[name];
    sp[name]->init(); st[name]->init();
}

template<>
void Fields<TF>::init_diagnostic_field(const std::string& name, const std::string& longname,
        const std::string& unit, const std::string& group, const std::array<int,3>& loc)
{
    sd[name] = std::make_shared<Field3d<TF>>(master, grid, name, longname, unit, group, loc);
    a[name] = sd[name];
}

template<>
std::shared_ptr<Field3d<TF>> Fields<TF>::get_tmp()
{
    auto& gd = grid.get_grid_data();
    auto f = std::make_shared<Field3d<TF>>(master, grid, "tmp", "", "", "", gd.sloc);
    f->init();
    return f;
}

template<> void Fields<TF>::release_tmp(std::shared_ptr<Field3d<TF>>& f) { f.reset(); }

// ---------------------------------------------------------------------------
// Statistics and output classes: no-ops (Stats::calc_tend is a no-op unless
// tendency statistics are on, src/stats.cxx:1810-1813).
// ---------------------------------------------------------------------------
template<> void Stats<TF>::add_tendency(const Field3d<TF>&, const std::string&, const std::string&, const std::string&, const std::string&) {}
template<> void Stats<TF>::add_profs(const Field3d<TF>&, const std::string&, std::vector<std::string>, const std::string&) {}
template<> void Stats<TF>::add_time_series(const std::string&, const std::string&, const std::string&, const std::string&, Stats_whitelist_type) {}
template<> void Stats<TF>::calc_stats(const std::string&, const Field3d<TF>&, const TF, const TF) {}
template<> void Stats<TF>::calc_stats_2d(const std::string&, const std::vector<TF>&, const TF) {}
template<> void Stats<TF>::calc_tend(Field3d<TF>&, const std::string&) {}
template<> void Column<TF>::add_time_series(std::string, std::string, std::string) {}
template<> void Column<TF>::calc_time_series(std::string, const TF* const, const TF) {}
template<> int Cross<TF>::cross_plane(TF*, const TF, std::string, int) { return 0; }
template<> std::vector<std::string> Cross<TF>::get_enabled_variables(const std::vector<std::string>&) { return {}; }

// ---------------------------------------------------------------------------
// Module base classes: constructors after src/advec.cxx:38-44,
// src/diff.cxx:43-52, src/pres.cxx:41-56, src/thermo.cxx:38-46.
// ---------------------------------------------------------------------------
template<>
Advec<TF>::Advec(Master& m, Grid<TF>& g, Fields<TF>& f, Input& input) :
    master(m), grid(g), fields(f), field3d_operators(master, grid, fields), cflmin(1.E-5)
{
    cflmax = input.get_item<TF>("advec", "cflmax", "", 1.);
}
template<> Advec<TF>::~Advec() {}

template<>
Diff<TF>::Diff(Master& m, Grid<TF>& g, Fields<TF>& f, Boundary<TF>& b, Input&) :
    master(m), grid(g), fields(f), boundary(b) {}
template<> Diff<TF>::~Diff() {}

template<>
Pres<TF>::Pres(Master& m, Grid<TF>& g, Fields<TF>& f, FFT<TF>& fft_in, Input&) :
    master(m), grid(g), fields(f), fft(fft_in), field3d_operators(master, grid, fields) {}
template<> Pres<TF>::~Pres() {}

template<>
Thermo<TF>::Thermo(Master& m, Grid<TF>& g, Fields<TF>& f, Input&) : master(m), grid(g), fields(f) {}
template<> Thermo<TF>::~Thermo() {}
template<> Thermo_type Thermo<TF>::get_switch() { return swthermo; }

// ---------------------------------------------------------------------------
// FFT: the serial branch of src/fft.cxx:337-452 (x transforms of all rows,
// then y transforms with stride iblock; inverse y then /jtot, inverse x then
// /itot into tmp1), with the oracle's halfcomplex transforms in place of FFTW.
//
// The inverse evaluates the mean mode (kx = ky = 0) of each level apart: the
// mode is set aside and zeroed, the other modes are transformed, and the
// level's mean (X_00/jtot)/itot is added to every point at the end.  That is
// the same unnormalised inverse transform; it only keeps the large
// hydrostatic part of the pressure out of the butterflies, whose round-off
// (eps times the mean, at every point) would otherwise depend on the order
// of the radix passes.  FFTW's own rounding is not reproducible here anyway.
// ---------------------------------------------------------------------------
template<> FFT<TF>::FFT(Master& m, Grid<TF>& g) : master(m), grid(g), transpose(m, g)
{
    has_fftw_plan = false;
    fftini = fftouti = fftinj = fftoutj = nullptr;
}
template<> FFT<TF>::~FFT() {}
template<> void FFT<TF>::init() {}
template<> void FFT<TF>::load() {}
template<> void FFT<TF>::save() {}

template<>
void FFT<TF>::exec_forward(TF* const restrict data, TF* const restrict)
{
    auto& gd = grid.get_grid_data();
    orcfft_r2hc(gd.itot, gd.jmax*gd.kblock, data, 1, gd.itot);
    for (int k=0; k<gd.kblock; ++k)
        orcfft_r2hc(gd.jtot, gd.iblock, data + (long)k*gd.iblock*gd.jtot, gd.iblock, 1);
}

template<>
void FFT<TF>::exec_backward(TF* const restrict data, TF* const restrict tmp1)
{
    auto& gd = grid.get_grid_data();
    const long n = (long)gd.itot*gd.jtot*gd.ktot;
    const long nlev = (long)gd.iblock*gd.jtot;
    std::vector<TF> mean(gd.kblock);
    for (int k=0; k<gd.kblock; ++k)
    {
        mean[k] = (data[k*nlev] / gd.jtot) / gd.itot;
        data[k*nlev] = TF(0);
    }
    for (int k=0; k<gd.kblock; ++k)
        orcfft_hc2r(gd.jtot, gd.iblock, data + (long)k*nlev, gd.iblock, 1);
    for (long q=0; q<n; ++q) data[q] = data[q] / gd.jtot;
    orcfft_hc2r(gd.itot, gd.jmax*gd.kblock, data, 1, gd.itot);
    for (long q=0; q<n; ++q) tmp1[q] = data[q] / gd.itot + mean[q / nlev];
}

// ---------------------------------------------------------------------------
// Boundary base class, src/boundary.cxx:156-1023 (2nd-order parts).
// ---------------------------------------------------------------------------
namespace
{
    // src/boundary.cxx:50-100
    void set_bc(TF* a, TF* agrad, TF* aflux, Boundary_type sw, TF aval, TF visc, TF offset,
                int n, bool set_flux_grad)
    {
        if (sw == Boundary_type::Dirichlet_type)
            for (int q=0; q<n; ++q) a[q] = aval - offset;
        else if (sw == Boundary_type::Neumann_type)
            for (int q=0; q<n; ++q) { agrad[q] = aval; if (set_flux_grad) aflux[q] = -aval*visc; }
        else if (sw == Boundary_type::Flux_type)
            for (int q=0; q<n; ++q) { aflux[q] = aval; if (set_flux_grad) agrad[q] = -aval/visc; }
    }

    // src/boundary.cxx:700-760
    void ghost_bot_2nd(TF* a, const TF* dzh, Boundary_type t, const TF* abot, const TF* agradbot,
                       int kstart, int icells, int jcells, int ijcells)
    {
        for (int j=0; j<jcells; ++j)
            for (int i=0; i<icells; ++i)
            {
                const int ij = i + j*icells;
                const int ijk = ij + kstart*ijcells;
                if (t == Boundary_type::Dirichlet_type)
                    a[ijk-ijcells] = TF(2.)*abot[ij] - a[ijk];
                else if (t == Boundary_type::Neumann_type || t == Boundary_type::Flux_type)
                    a[ijk-ijcells] = -agradbot[ij]*dzh[kstart] + a[ijk];
            }
    }

    void ghost_top_2nd(TF* a, const TF* dzh, Boundary_type t, const TF* atop, const TF* agradtop,
                       int kend, int icells, int jcells, int ijcells)
    {
        for (int j=0; j<jcells; ++j)
            for (int i=0; i<icells; ++i)
            {
                const int ij = i + j*icells;
                const int ijk = ij + (kend-1)*ijcells;
                if (t == Boundary_type::Dirichlet_type)
                    a[ijk+ijcells] = TF(2.)*atop[ij] - a[ijk];
                else if (t == Boundary_type::Neumann_type || t == Boundary_type::Flux_type)
                    a[ijk+ijcells] = agradtop[ij]*dzh[kend] + a[ijk];
            }
    }

    Boundary_type bc_from_string(const std::string& s, bool momentum)
    {
        if (momentum)
        {
            if (s == "noslip") return Boundary_type::Dirichlet_type;
            if (s == "freeslip" || s == "neumann") return Boundary_type::Neumann_type;
        }
        else
        {
            if (s == "dirichlet") return Boundary_type::Dirichlet_type;
            if (s == "neumann") return Boundary_type::Neumann_type;
            if (s == "flux") return Boundary_type::Flux_type;
        }
        throw std::runtime_error(s + " is an illegal boundary type");
    }
}

template<>
Boundary<TF>::Boundary(Master& m, Grid<TF>& g, Soil_grid<TF>& sg, Fields<TF>& f, Input& input) :
    master(m), grid(g), soil_grid(sg), fields(f),
    boundary_cyclic(master, grid), field3d_io(master, grid), boundary_outflow(master, grid, input)
{
    swboundary = "default";
    swtimedep_outflow = false;
    swtimedep_sbot_2d = false;
}

template<> Boundary<TF>::~Boundary() { sbc.clear(); }
template<> std::string Boundary<TF>::get_switch() { return swboundary; }

// src/boundary.cxx:185-262
template<>
void Boundary<TF>::process_bcs(Input& input)
{
    mbcbot = bc_from_string(input.get_item<std::string>("boundary", "mbcbot", ""), true);
    mbctop = bc_from_string(input.get_item<std::string>("boundary", "mbctop", ""), true);
    ubot = input.get_item<TF>("boundary", "ubot", "", 0.);
    utop = input.get_item<TF>("boundary", "utop", "", 0.);
    vbot = input.get_item<TF>("boundary", "vbot", "", 0.);
    vtop = input.get_item<TF>("boundary", "vtop", "", 0.);
    for (auto& it : fields.sp)
    {
        sbc.emplace(it.first, Field3dBc<TF>());
        sbc.at(it.first).bcbot = bc_from_string(input.get_item<std::string>("boundary", "sbcbot", it.first), false);
        sbc.at(it.first).bctop = bc_from_string(input.get_item<std::string>("boundary", "sbctop", it.first), false);
        sbc.at(it.first).bot = input.get_item<TF>("boundary", "sbot", it.first);
        sbc.at(it.first).top = input.get_item<TF>("boundary", "stop", it.first);
    }
}

template<> void Boundary<TF>::init(Input& input, Thermo<TF>&, const Sim_mode) { process_bcs(input); boundary_cyclic.init(); }
template<> void Boundary<TF>::process_time_dependent(Input&, Netcdf_handle&, Timeloop<TF>&) {}
template<> void Boundary<TF>::process_inflow(Input&, Netcdf_handle&) {}
template<> void Boundary<TF>::create_cold_start(Netcdf_handle&) {}
template<> void Boundary<TF>::create(Input&, Netcdf_handle&, Stats<TF>&, Column<TF>&, Cross<TF>&, Timeloop<TF>&) {}
template<> void Boundary<TF>::update_time_dependent(Timeloop<TF>&) {}
template<> void Boundary<TF>::exec(Thermo<TF>&, Radiation<TF>&, Microphys<TF>&, Timeloop<TF>&) {}
template<> void Boundary<TF>::exec_stats(Stats<TF>&) {}
template<> void Boundary<TF>::exec_column(Column<TF>&) {}
template<> void Boundary<TF>::set_ghost_cells_w(Boundary_w_type) {}
template<> void Boundary<TF>::update_slave_bcs() {}
namespace { std::vector<TF> empty_vec; }
template<> const std::vector<TF>& Boundary<TF>::get_z0m() const { throw std::runtime_error("no z0m"); return empty_vec; }
template<> const std::vector<TF>& Boundary<TF>::get_dudz() const { throw std::runtime_error("no dudz"); return empty_vec; }
template<> const std::vector<TF>& Boundary<TF>::get_dvdz() const { throw std::runtime_error("no dvdz"); return empty_vec; }
template<> const std::vector<TF>& Boundary<TF>::get_dbdz() const { throw std::runtime_error("no dbdz"); return empty_vec; }

// src/boundary.cxx:615-700 (non-timedependent, homogeneous branch)
template<>
void Boundary<TF>::set_values()
{
    auto& gd = grid.get_grid_data();
    const bool sfg = (swboundary == "default");
    const int n = gd.ijcells;
    auto& u = *fields.mp.at("u");
    auto& v = *fields.mp.at("v");
    set_bc(u.fld_bot.data(), u.grad_bot.data(), u.flux_bot.data(), mbcbot, ubot, fields.visc, gd.utrans, n, true);
    set_bc(v.fld_bot.data(), v.grad_bot.data(), v.flux_bot.data(), mbcbot, vbot, fields.visc, gd.vtrans, n, true);
    set_bc(u.fld_top.data(), u.grad_top.data(), u.flux_top.data(), mbctop, utop, fields.visc, gd.utrans, n, true);
    set_bc(v.fld_top.data(), v.grad_top.data(), v.flux_top.data(), mbctop, vtop, fields.visc, gd.vtrans, n, true);
    for (auto& it : fields.sp)
    {
        auto& s = *it.second;
        auto& bc = sbc.at(it.first);
        set_bc(s.fld_bot.data(), s.grad_bot.data(), s.flux_bot.data(), bc.bcbot, bc.bot, s.visc, 0., n, sfg);
        set_bc(s.fld_top.data(), s.grad_top.data(), s.flux_top.data(), bc.bctop, bc.top, s.visc, 0., n, sfg);
    }
}

// src/boundary.cxx:450-461
template<>
void Boundary<TF>::set_prognostic_cyclic_bcs()
{
    boundary_cyclic.exec(fields.mp.at("u")->fld.data());
    boundary_cyclic.exec(fields.mp.at("v")->fld.data());
    boundary_cyclic.exec(fields.mp.at("w")->fld.data());
    for (auto& it : fields.sp)
        boundary_cyclic.exec(it.second->fld.data());
}

// src/boundary.cxx:933-998 (second order)
template<>
void Boundary<TF>::set_ghost_cells()
{
    auto& gd = grid.get_grid_data();
    auto run = [&](Field3d<TF>& f, Boundary_type bot, Boundary_type top)
    {
        ghost_bot_2nd(f.fld.data(), gd.dzh.data(), bot, f.fld_bot.data(), f.grad_bot.data(),
                      gd.kstart, gd.icells, gd.jcells, gd.ijcells);
        ghost_top_2nd(f.fld.data(), gd.dzh.data(), top, f.fld_top.data(), f.grad_top.data(),
                      gd.kend, gd.icells, gd.jcells, gd.ijcells);
    };
    run(*fields.mp.at("u"), mbcbot, mbctop);
    run(*fields.mp.at("v"), mbcbot, mbctop);
    for (auto& it : fields.sp)
        run(*it.second, sbc.at(it.first).bcbot, sbc.at(it.first).bctop);
    update_slave_bcs();
}

template class Boundary<double>;

// ---------------------------------------------------------------------------
// Dry Boussinesq thermodynamics, restated from src/thermo_dry.cxx.
// ---------------------------------------------------------------------------
namespace ref_harness
{
    Thermo_dry_ref::Thermo_dry_ref(Master& m, Grid<TF>& g, Fields<TF>& f, Input& input, bool enabled) :
        Thermo<TF>(m, g, f, input)
    {
        swthermo = enabled ? Thermo_type::Dry : Thermo_type::Disabled;
        if (enabled)
        {
            auto& gd = grid.get_grid_data();
            // Boussinesq base state, src/thermo_dry.cxx:547-559
            const TF thref0 = input.get_item<TF>("thermo", "thref0", "");
            thref.assign(gd.kcells, thref0);
            threfh.assign(gd.kcells, thref0);
        }
    }
    Thermo_dry_ref::~Thermo_dry_ref() {}

    unsigned long Thermo_dry_ref::get_time_limit(unsigned long, double) { return Constants::ulhuge; }

    // src/thermo_dry.cxx:165-181, :610-627
    void Thermo_dry_ref::exec(const double, Stats<TF>&)
    {
        if (swthermo == Thermo_type::Disabled) return;
        auto& gd = grid.get_grid_data();
        TF* wt = fields.mt.at("w")->fld.data();
        const TF* th = fields.sp.at("th")->fld.data();
        for (int k=gd.kstart+1; k<gd.kend; ++k)
            for (int j=gd.jstart; j<gd.jend; ++j)
                for (int i=gd.istart; i<gd.iend; ++i)
                {
                    const int ijk = i + j*gd.icells + k*gd.ijcells;
                    wt[ijk] += Constants::grav<TF>/threfh[k] * (TF(0.5)*(th[ijk-gd.ijcells] + th[ijk]) - threfh[k]);
                }
    }

    // src/thermo_dry.cxx:64-75, :676-697 (N2 only)
    void Thermo_dry_ref::get_thermo_field(Field3d<TF>& fld, const std::string& name, const bool, const bool)
    {
        if (name != "N2") throw std::runtime_error("harness thermo only provides N2");
        auto& gd = grid.get_grid_data();
        const TF* th = fields.sp.at("th")->fld.data();
        for (int k=gd.kstart; k<gd.kend; ++k)
            for (int j=gd.jstart; j<gd.jend; ++j)
                for (int i=gd.istart; i<gd.iend; ++i)
                {
                    const int ijk = i + j*gd.icells + k*gd.ijcells;
                    fld.fld[ijk] = Constants::grav<TF>/thref[k]*TF(0.5)*(th[ijk+gd.ijcells] - th[ijk-gd.ijcells])*gd.dzi[k];
                }
    }

    // src/thermo_dry.cxx:133-147, :720-740
    void Thermo_dry_ref::get_buoyancy_surf(std::vector<TF>& b, std::vector<TF>& bbot, bool)
    {
        auto& gd = grid.get_grid_data();
        const TF* th = fields.sp.at("th")->fld.data();
        const TF* thbot = fields.sp.at("th")->fld_bot.data();
        for (int j=0; j<gd.jcells; ++j)
            for (int i=0; i<gd.icells; ++i)
            {
                const int ij = i + j*gd.icells;
                const int ijk = ij + gd.kstart*gd.ijcells;
                bbot[ij] = Constants::grav<TF>/threfh[gd.kstart] * (thbot[ij] - threfh[gd.kstart]);
                b[ijk]   = Constants::grav<TF>/thref [gd.kstart] * (th[ijk]   - thref [gd.kstart]);
            }
    }

    void Thermo_dry_ref::get_buoyancy_surf(std::vector<TF>&, std::vector<TF>&, std::vector<TF>&)
    { throw std::runtime_error("not on the hot path"); }

    // src/thermo_dry.cxx:150-162, :700-718
    void Thermo_dry_ref::get_buoyancy_fluxbot(std::vector<TF>& bfluxbot, bool)
    {
        auto& gd = grid.get_grid_data();
        const TF* flux = fields.sp.at("th")->flux_bot.data();
        for (int n=0; n<gd.ijcells; ++n)
            bfluxbot[n] = Constants::grav<TF>/threfh[gd.kstart]*flux[n];
    }

    void Thermo_dry_ref::get_temperature_bot(Field3d<TF>&, bool) { throw std::runtime_error("not on the hot path"); }
    void Thermo_dry_ref::get_prog_vars(std::vector<std::string>& list)
    { if (swthermo != Thermo_type::Disabled) list.push_back("th"); }
    void Thermo_dry_ref::get_radiation_fields(Field3d<TF>&, Field3d<TF>&, Field3d<TF>&, Field3d<TF>&, Field3d<TF>&) const
    { throw std::runtime_error("not on the hot path"); }
    void Thermo_dry_ref::get_radiation_fields(Field3d<TF>&, Field3d<TF>&, Field3d<TF>&, Field3d<TF>&, Field3d<TF>&, Field3d<TF>&) const
    { throw std::runtime_error("not on the hot path"); }
    void Thermo_dry_ref::get_radiation_columns(Field3d<TF>&, std::vector<int>&, std::vector<int>&) const
    { throw std::runtime_error("not on the hot path"); }
    void Thermo_dry_ref::get_land_surface_fields(std::vector<TF>&, std::vector<TF>&, std::vector<TF>&, std::vector<TF>&, std::vector<TF>&)
    { throw std::runtime_error("not on the hot path"); }
    const std::vector<TF>& Thermo_dry_ref::get_basestate_vector(std::string name) const
    {
        if (name == "th") return thref;
        if (name == "thh") return threfh;
        throw std::runtime_error("not on the hot path");
    }
    // src/thermo_dry.cxx:780-784
    TF Thermo_dry_ref::get_db_ref() const
    {
        auto& gd = grid.get_grid_data();
        return Constants::grav<TF>/thref[gd.kstart]*(thref[gd.kstart] - threfh[gd.kstart]);
    }
}

// ---------------------------------------------------------------------------
// Initial profiles for Buffer::create (src/buffer.cxx:130-150), in place of
// the "init" group of the case's NetCDF input.
// ---------------------------------------------------------------------------
namespace
{
    std::map<std::string, std::vector<double>> g_init_profiles;
}

void ref_harness::set_init_profile(const std::string& name, const std::vector<double>& prof)
{
    g_init_profiles[name] = prof;
}

Netcdf_group& Netcdf_handle::get_group(const std::string&)
{
    // Never dereferenced: get_variable below ignores the handle.
    return *reinterpret_cast<Netcdf_group*>(this);
}

// The first prod(count) values of `values` receive the variable (the vector is
// not resized), or zeros when it does not exist
// (src/netcdf_interface.cxx:647-692).
template<>
void Netcdf_handle::get_variable<double>(std::vector<double>& values, const std::string& name,
                                         const std::vector<int>&, const std::vector<int>& count, const bool)
{
    size_t n = 1;
    for (int c : count) n *= size_t(c);
    auto it = g_init_profiles.find(name);
    for (size_t q=0; q<n; ++q)
        values[q] = it != g_init_profiles.end() && q < it->second.size() ? it->second[q] : 0.;
}
