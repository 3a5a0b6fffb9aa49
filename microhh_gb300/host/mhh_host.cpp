// mhh_host.cpp -- implementation of the C++ host layer (see mhh_host.h) and
// its C entry points mhh_model_* (include/mhh_model.h).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <cstdio>
#include <sstream>

#include <cuda_runtime.h>

#include "mhh_host.h"
#include "mhh_model.h"

namespace mhh_host
{
    void check(int rc, const char* what)
    {
        if (rc == MHH_ERR_NONFINITE)
            throw Nonfinite_error(std::string(what) + ": " + mhh_last_error());
        if (rc != MHH_OK)
            throw std::runtime_error(std::string(what) + ": " + mhh_last_error());
    }

    static void cuda_check(cudaError_t e, const char* what)
    {
        if (e != cudaSuccess)
            throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
    }

    // ---------------------------------------------------------------------
    // Input: [group] headers, key=value and key[subkey]=value lines, '#'
    // comments, lists split on ',' (src/input.cxx:77-222, src/input.cxx:366-430).
    // ---------------------------------------------------------------------
    static std::string trim(const std::string& s)
    {
        const size_t a = s.find_first_not_of(" \t\r");
        if (a == std::string::npos) return "";
        const size_t b = s.find_last_not_of(" \t\r");
        return s.substr(a, b - a + 1);
    }

    Input::Input(const std::string& text)
    {
        std::istringstream ss(text);
        std::string line, group;
        int lineno = 0;
        while (std::getline(ss, line))
        {
            ++lineno;
            const size_t hash = line.find('#');
            if (hash != std::string::npos) line = line.substr(0, hash);
            line = trim(line);
            if (line.empty()) continue;
            if (line.front() == '[')
            {
                if (line.back() != ']') throw std::runtime_error("line " + std::to_string(lineno) + ": bad group header");
                group = trim(line.substr(1, line.size() - 2));
                continue;
            }
            const size_t eq = line.find('=');
            if (eq == std::string::npos || group.empty())
                throw std::runtime_error("line " + std::to_string(lineno) + ": expected key=value in a [group]");
            std::string key = trim(line.substr(0, eq));
            const std::string val = trim(line.substr(eq + 1));
            std::string sub;
            const size_t lb = key.find('[');
            if (lb != std::string::npos)
            {
                const size_t rb = key.find(']', lb);
                if (rb == std::string::npos) throw std::runtime_error("line " + std::to_string(lineno) + ": bad subkey");
                sub = trim(key.substr(lb + 1, rb - lb - 1));
                key = trim(key.substr(0, lb));
            }
            items[group][key][sub] = std::make_pair(val, false);
        }
    }

    bool Input::find(const std::string& g, const std::string& k, const std::string& s, std::string& out)
    {
        auto ig = items.find(g);
        if (ig == items.end()) return false;
        auto ik = ig->second.find(k);
        if (ik == ig->second.end()) return false;
        auto is = ik->second.find(s);
        if (is == ik->second.end()) is = ik->second.find("");
        if (is == ik->second.end()) return false;
        is->second.second = true;
        out = is->second.first;
        return true;
    }

    template<typename T> static T parse(const std::string& v, const std::string& what);
    template<> int parse<int>(const std::string& v, const std::string& w)
    { try { size_t p; int r = std::stoi(v, &p); if (p != v.size()) throw 0; return r; } catch (...) { throw std::runtime_error("item " + w + " is not an integer: " + v); } }
    template<> double parse<double>(const std::string& v, const std::string& w)
    { try { size_t p; double r = std::stod(v, &p); if (p != v.size()) throw 0; return r; } catch (...) { throw std::runtime_error("item " + w + " is not a number: " + v); } }
    template<> std::string parse<std::string>(const std::string& v, const std::string&) { return v; }
    template<> bool parse<bool>(const std::string& v, const std::string& w)
    {
        if (v == "1" || v == "true" || v == "True") return true;
        if (v == "0" || v == "false" || v == "False") return false;
        throw std::runtime_error("item " + w + " is not a bool: " + v);
    }

    template<typename T>
    T Input::get_item(const std::string& g, const std::string& k, const std::string& s)
    {
        std::string v;
        if (!find(g, k, s, v))
            throw std::runtime_error("item [" + g + "][" + k + "]" + (s.empty() ? "" : "[" + s + "]") + " does not exist");
        return parse<T>(v, g + "." + k);
    }

    template<typename T>
    T Input::get_item(const std::string& g, const std::string& k, const std::string& s, const T def)
    {
        std::string v;
        if (!find(g, k, s, v)) return def;
        return parse<T>(v, g + "." + k);
    }

    std::vector<std::string> Input::get_list(const std::string& g, const std::string& k, const std::string& s,
                                             const std::vector<std::string>& def)
    {
        std::string v;
        if (!find(g, k, s, v)) return def;
        std::vector<std::string> out;
        std::string tok;
        std::istringstream ss(v);
        while (std::getline(ss, tok, ','))
        {
            const size_t b = tok.find_first_not_of(" \t"), e = tok.find_last_not_of(" \t");
            if (b != std::string::npos) out.push_back(tok.substr(b, e - b + 1));
        }
        return out;
    }

    std::vector<std::string> Input::unused_items() const
    {
        std::vector<std::string> out;
        for (auto& g : items) for (auto& k : g.second) for (auto& s : k.second)
            if (!s.second.second) out.push_back(g.first + "." + k.first + (s.first.empty() ? "" : "[" + s.first + "]"));
        return out;
    }

    template int Input::get_item<int>(const std::string&, const std::string&, const std::string&);
    template double Input::get_item<double>(const std::string&, const std::string&, const std::string&);
    template bool Input::get_item<bool>(const std::string&, const std::string&, const std::string&);
    template std::string Input::get_item<std::string>(const std::string&, const std::string&, const std::string&);
    template int Input::get_item<int>(const std::string&, const std::string&, const std::string&, const int);
    template double Input::get_item<double>(const std::string&, const std::string&, const std::string&, const double);
    template bool Input::get_item<bool>(const std::string&, const std::string&, const std::string&, const bool);
    template std::string Input::get_item<std::string>(const std::string&, const std::string&, const std::string&, const std::string);

    static int momentum_bc(const std::string& s, bool top)
    {
        if (s == "noslip") return MHH_BC_DIRICHLET;
        if (s == "freeslip" || s == "neumann") return MHH_BC_NEUMANN;
        throw std::runtime_error(s + " is an illegal value for " + (top ? "mbctop" : "mbcbot"));
    }

    static int scalar_bc(const std::string& s, bool top)
    {
        if (s == "dirichlet") return MHH_BC_DIRICHLET;
        if (s == "neumann") return MHH_BC_NEUMANN;
        if (s == "flux") return MHH_BC_FLUX;
        throw std::runtime_error(s + " is an illegal value for " + (top ? "sbctop" : "sbcbot"));
    }

    // ---------------------------------------------------------------------
    // Grid
    // ---------------------------------------------------------------------
    template<typename TF>
    Grid<TF>::Grid(Input& in, int igc, int kgc)
    {
        desc.itot = in.get_item<int>("grid", "itot", "");
        desc.jtot = in.get_item<int>("grid", "jtot", "");
        desc.ktot = in.get_item<int>("grid", "ktot", "");
        desc.xsize = in.get_item<double>("grid", "xsize", "");
        desc.ysize = in.get_item<double>("grid", "ysize", "");
        desc.zsize = in.get_item<double>("grid", "zsize", "");
        const std::string order = in.get_item<std::string>("grid", "swspatialorder", "", "2");
        if (order != "2") throw std::runtime_error("only swspatialorder=2 is on this path");
        desc.igc = igc; desc.jgc = igc; desc.kgc = kgc;
        std::memset(&phys, 0, sizeof(phys));
        phys.visc = in.get_item<double>("fields", "visc", "");
        phys.svisc = in.get_item<double>("fields", "svisc", "", phys.visc);
        phys.cs = in.get_item<double>("diff", "cs", "", 0.23);
        phys.tpr = in.get_item<double>("diff", "tPr", "", 1./3.);
        phys.dnmax = in.get_item<double>("diff", "dnmax", "", 0.4);
        phys.swmason = in.get_item<bool>("diff", "swmason", "", true) ? 1 : 0;
        phys.cflmax = in.get_item<double>("advec", "cflmax", "", 1.);
        const std::string swthermo = in.get_item<std::string>("thermo", "swthermo", "", "0");
        phys.thermo = swthermo == "dry" ? 1 : 0;
        if (swthermo != "dry" && swthermo != "0") throw std::runtime_error("swthermo must be dry or 0 on this path");
        phys.thref0 = phys.thermo ? in.get_item<double>("thermo", "thref0", "") : 300.;
        if (phys.thermo && in.get_item<std::string>("thermo", "swbasestate", "", "boussinesq") != "boussinesq")
            throw std::runtime_error("only swbasestate=boussinesq is on this path");
        in.get_item<double>("thermo", "pbot", "", 1.e5);
        const std::string swb = in.get_item<std::string>("boundary", "swboundary", "", "default");
        if (swb != "default" && swb != "surface") throw std::runtime_error("swboundary must be default or surface");
        phys.surface = swb == "surface" ? 1 : 0;
        phys.z0m = phys.surface ? in.get_item<double>("boundary", "z0m", "") : 0.;
        phys.z0h = phys.surface ? in.get_item<double>("boundary", "z0h", "") : 0.;
        std::memset(&gd, 0, sizeof(gd));
    }

    template<typename TF>
    Grid<TF>::~Grid() { if (ctx_) mhh_ctx_destroy(ctx_); }

    template<typename TF>
    void Grid<TF>::create(const std::vector<double>& z)
    {
        if ((int)z.size() != desc.ktot) throw std::runtime_error("z must have ktot levels");
        if (z.back() > desc.zsize) throw std::runtime_error("Highest grid point is above prescribed zsize");
        check(mhh_ctx_create(&desc, z.data(), sizeof(TF) == 8 ? MHH_FP64 : MHH_FP32, &phys, &ctx_), "mhh_ctx_create");
        check(mhh_ctx_get_grid(ctx_, &gd), "mhh_ctx_get_grid");
    }

    template<typename TF>
    std::vector<double> Grid<TF>::profile(const std::string& name) const
    {
        std::vector<double> v(gd.kcells);
        check(mhh_ctx_get_profile(ctx_, name.c_str(), v.data()), "profile");
        return v;
    }

    // ---------------------------------------------------------------------
    // Fields
    // ---------------------------------------------------------------------
    // Stream-ordered allocation on the model's set-up stream: creating and
    // destroying a model does not synchronise the work of other models.
    template<typename TF>
    Field3d<TF>::Field3d(const std::string& n, long long ncells, int ijcells, cudaStream_t s) : name(n), alloc_stream(s)
    {
        cuda_check(cudaMallocAsync((void**)&fld_g, sizeof(TF)*ncells, s), "cudaMallocAsync field");
        cuda_check(cudaMemsetAsync(fld_g, 0, sizeof(TF)*ncells, s), "cudaMemsetAsync field");
        TF** two_d[] = {&fld_bot_g, &fld_top_g, &grad_bot_g, &grad_top_g, &flux_bot_g, &flux_top_g};
        for (TF** p : two_d)
        {
            cuda_check(cudaMallocAsync((void**)p, sizeof(TF)*ijcells, s), "cudaMallocAsync boundary array");
            cuda_check(cudaMemsetAsync(*p, 0, sizeof(TF)*ijcells, s), "cudaMemsetAsync boundary array");
        }
    }

    template<typename TF>
    Field3d<TF>::~Field3d()
    {
        TF* ps[] = {fld_g, fld_bot_g, fld_top_g, grad_bot_g, grad_top_g, flux_bot_g, flux_top_g};
        for (TF* p : ps) if (p) cudaFreeAsync(p, alloc_stream);
    }

    template<typename TF>
    Fields<TF>::Fields(Grid<TF>& g, Input& in, bool with_scalar, bool with_evisc) : grid(g)
    {
        const auto& gd = g.get_grid_data();
        visc = g.phys.visc;
        svisc = g.phys.svisc;
        cuda_check(cudaStreamCreateWithFlags(&setup, cudaStreamNonBlocking), "stream");
        auto make = [&](const std::string& n) { return std::make_shared<Field3d<TF>>(n, gd.ncells, gd.ijcells, setup); };
        for (const char* n : {"u", "v", "w"}) { mp[n] = make(n); mt[n] = make(std::string(n) + "t"); mp[n]->visc = visc; }
        if (with_scalar) { sp["th"] = make("th"); st["th"] = make("tht"); sp["th"]->visc = svisc; }
        sd["p"] = make("p");
        if (with_evisc) sd["evisc"] = make("evisc");
        (void)in;
        // The allocations and their zeroing are ordered on the set-up stream
        // only; every later use (host copies on the default stream, kernels
        // on the model's stream) must find them done.
        cuda_check(cudaStreamSynchronize(setup), "field set-up");
    }

    template<typename TF>
    Fields<TF>::~Fields()
    {
        mp.clear(); mt.clear(); sp.clear(); st.clear(); sd.clear();
        if (setup)
        {
            cudaStreamSynchronize(setup);
            cudaStreamDestroy(setup);
        }
    }

    template<typename TF>
    mhh_fields Fields<TF>::dev() const
    {
        mhh_fields f;
        std::memset(&f, 0, sizeof(f));
        f.u = mp.at("u")->fld_g; f.v = mp.at("v")->fld_g; f.w = mp.at("w")->fld_g;
        f.ut = mt.at("u")->fld_g; f.vt = mt.at("v")->fld_g; f.wt = mt.at("w")->fld_g;
        if (sp.count("th")) { f.s = sp.at("th")->fld_g; f.st = st.at("th")->fld_g; }
        if (sd.count("evisc")) f.evisc = sd.at("evisc")->fld_g;
        f.p = sd.at("p")->fld_g;
        return f;
    }

    template<typename TF>
    mhh_bcfields Fields<TF>::bc() const
    {
        mhh_bcfields b;
        std::memset(&b, 0, sizeof(b));
        const auto& u = *mp.at("u"); const auto& v = *mp.at("v");
        b.u_bot = u.fld_bot_g; b.u_top = u.fld_top_g; b.u_gradbot = u.grad_bot_g; b.u_gradtop = u.grad_top_g;
        b.u_fluxbot = u.flux_bot_g; b.u_fluxtop = u.flux_top_g;
        b.v_bot = v.fld_bot_g; b.v_top = v.fld_top_g; b.v_gradbot = v.grad_bot_g; b.v_gradtop = v.grad_top_g;
        b.v_fluxbot = v.flux_bot_g; b.v_fluxtop = v.flux_top_g;
        if (sp.count("th"))
        {
            const auto& s = *sp.at("th");
            b.s_bot = s.fld_bot_g; b.s_top = s.fld_top_g; b.s_gradbot = s.grad_bot_g; b.s_gradtop = s.grad_top_g;
            b.s_fluxbot = s.flux_bot_g; b.s_fluxtop = s.flux_top_g;
        }
        return b;
    }

    template<typename TF>
    Field3d<TF>* Fields<TF>::by_name(const std::string& n) const
    {
        if (mp.count(n)) return mp.at(n).get();
        if (sp.count(n)) return sp.at(n).get();
        if (sd.count(n)) return sd.at(n).get();
        if (n.size() > 1 && n.back() == 't')
        {
            const std::string b = n.substr(0, n.size() - 1);
            if (mt.count(b)) return mt.at(b).get();
            if (st.count(b)) return st.at(b).get();
        }
        throw std::runtime_error("unknown field " + n);
    }

    template<typename TF>
    double Fields<TF>::offset(const std::string& name) const
    {
        if (name != "th") return 0.;
        double off = 0.;
        check(mhh_ctx_scalar_offset(grid.ctx(), &off), "scalar_offset");
        return off;
    }

    template<typename TF>
    void Fields<TF>::set_from_host(const std::string& name, const double* data)
    {
        Field3d<TF>* f = by_name(name);
        const long long n = grid.get_grid_data().ncells;
        const double off = offset(name);
        if (sizeof(TF) == 8 && off == 0.)
            cuda_check(cudaMemcpy(f->fld_g, data, sizeof(double)*n, cudaMemcpyHostToDevice), "set field");
        else
        {
            // The difference is taken in double and rounded once.
            std::vector<TF> tmp(n);
            for (long long q=0; q<n; ++q) tmp[q] = TF(data[q] - off);
            cuda_check(cudaMemcpy(f->fld_g, tmp.data(), sizeof(TF)*n, cudaMemcpyHostToDevice), "set field");
        }
    }

    template<typename TF>
    void Fields<TF>::get_to_host(const std::string& name, double* data) const
    {
        Field3d<TF>* f = by_name(name);
        const long long n = grid.get_grid_data().ncells;
        const double off = offset(name);
        if (sizeof(TF) == 8 && off == 0.)
            cuda_check(cudaMemcpy(data, f->fld_g, sizeof(double)*n, cudaMemcpyDeviceToHost), "get field");
        else
        {
            std::vector<TF> tmp(n);
            cuda_check(cudaMemcpy(tmp.data(), f->fld_g, sizeof(TF)*n, cudaMemcpyDeviceToHost), "get field");
            for (long long q=0; q<n; ++q) data[q] = double(tmp[q]) + off;
        }
    }

    template<typename TF>
    void Fields<TF>::set_native(const std::string& name, const void* data, cudaStream_t s)
    {
        Field3d<TF>* f = by_name(name);
        cuda_check(cudaMemcpyAsync(f->fld_g, data, sizeof(TF)*grid.get_grid_data().ncells, cudaMemcpyHostToDevice, s),
                   "set field");
        const double off = offset(name);
        if (off != 0.) check(mhh_field_shift(grid.ctx(), f->fld_g, -off, s), "field_shift");
    }

    template<typename TF>
    void Fields<TF>::get_native(const std::string& name, void* data, cudaStream_t s) const
    {
        Field3d<TF>* f = by_name(name);
        const long long n = grid.get_grid_data().ncells;
        const double off = offset(name);
        if (off == 0.)
        {
            cuda_check(cudaMemcpyAsync(data, f->fld_g, sizeof(TF)*n, cudaMemcpyDeviceToHost, s), "get field");
            return;
        }
        // Native values are physical: the offset is added (rounded to the
        // field precision) on the device, in a stream-ordered scratch copy,
        // so that the copy to the host stays one DMA transfer.
        void* tmp = nullptr;
        cuda_check(cudaMallocAsync(&tmp, sizeof(TF)*n, s), "get field");
        try
        {
            cuda_check(cudaMemcpyAsync(tmp, f->fld_g, sizeof(TF)*n, cudaMemcpyDeviceToDevice, s), "get field");
            check(mhh_field_shift(grid.ctx(), tmp, off, s), "field_shift");
            cuda_check(cudaMemcpyAsync(data, tmp, sizeof(TF)*n, cudaMemcpyDeviceToHost, s), "get field");
        }
        catch (...)
        {
            cudaFreeAsync(tmp, s);
            throw;
        }
        cuda_check(cudaFreeAsync(tmp, s), "get field");
    }

    // ---------------------------------------------------------------------
    // Boundary, src/boundary.cxx:185-262 (process_bcs), :615-700 (set_values)
    // and src/boundary_surface.cxx:755-790 (surface override).
    // ---------------------------------------------------------------------
    template<typename TF>
    Boundary<TF>::Boundary(Grid<TF>& g, Fields<TF>& f, Input& in) : grid(g), fields(f)
    {
        swboundary = in.get_item<std::string>("boundary", "swboundary", "", "default");
        mbcbot = momentum_bc(in.get_item<std::string>("boundary", "mbcbot", ""), false);
        mbctop = momentum_bc(in.get_item<std::string>("boundary", "mbctop", ""), true);
        ubot = in.get_item<double>("boundary", "ubot", "", 0.);
        utop = in.get_item<double>("boundary", "utop", "", 0.);
        vbot = in.get_item<double>("boundary", "vbot", "", 0.);
        vtop = in.get_item<double>("boundary", "vtop", "", 0.);
        sbcbot = sbctop = MHH_BC_NEUMANN;
        sbot = stop = 0.;
        if (fields.sp.count("th"))
        {
            sbcbot = scalar_bc(in.get_item<std::string>("boundary", "sbcbot", "th"), false);
            sbctop = scalar_bc(in.get_item<std::string>("boundary", "sbctop", "th"), true);
            sbot = in.get_item<double>("boundary", "sbot", "th");
            stop = in.get_item<double>("boundary", "stop", "th");
        }
        if (swboundary == "surface")
        {
            if (mbcbot != MHH_BC_DIRICHLET) throw std::runtime_error("the surface model needs mbcbot=noslip on this path");
            if (fields.sp.count("th") && sbcbot == MHH_BC_NEUMANN)
                throw std::runtime_error("Fixed Gradient bc is not supported in surface model");
        }
    }

    template<typename TF>
    void Boundary<TF>::set_values()
    {
        mhh_ctx* c = grid.ctx();
        const bool sfg = swboundary == "default";
        auto& u = *fields.mp.at("u"); auto& v = *fields.mp.at("v");
        check(mhh_boundary_set_bc(c, u.fld_bot_g, u.grad_bot_g, u.flux_bot_g, mbcbot, ubot, fields.visc, 1, 0), "set_bc");
        check(mhh_boundary_set_bc(c, v.fld_bot_g, v.grad_bot_g, v.flux_bot_g, mbcbot, vbot, fields.visc, 1, 0), "set_bc");
        check(mhh_boundary_set_bc(c, u.fld_top_g, u.grad_top_g, u.flux_top_g, mbctop, utop, fields.visc, 1, 0), "set_bc");
        check(mhh_boundary_set_bc(c, v.fld_top_g, v.grad_top_g, v.flux_top_g, mbctop, vtop, fields.visc, 1, 0), "set_bc");
        if (fields.sp.count("th"))
        {
            auto& s = *fields.sp.at("th");
            // A Dirichlet value is a temperature, stored with the scalar's
            // offset; gradients and fluxes are unchanged by it.
            const double off = fields.offset("th");
            const double vb = sbcbot == MHH_BC_DIRICHLET ? sbot - off : sbot;
            const double vt = sbctop == MHH_BC_DIRICHLET ? stop - off : stop;
            check(mhh_boundary_set_bc(c, s.fld_bot_g, s.grad_bot_g, s.flux_bot_g, sbcbot, vb, s.visc, sfg, 0), "set_bc");
            check(mhh_boundary_set_bc(c, s.fld_top_g, s.grad_top_g, s.flux_top_g, sbctop, vt, s.visc, sfg, 0), "set_bc");
        }
        if (swboundary == "surface")
        {
            check(mhh_boundary_set_bc(c, u.fld_bot_g, u.grad_bot_g, u.flux_bot_g, MHH_BC_DIRICHLET, ubot, fields.visc, 0, 0), "set_bc");
            check(mhh_boundary_set_bc(c, v.fld_bot_g, v.grad_bot_g, v.flux_bot_g, MHH_BC_DIRICHLET, vbot, fields.visc, 0, 0), "set_bc");
            check(mhh_boundary_surface_init(c, fields.sp.count("th") ? sbcbot : MHH_BC_FLUX), "surface_init");
        }
        // The BC kernels ran on the legacy stream and the fields were
        // allocated on the fields' set-up stream; wait for both only.
        cuda_check(cudaStreamSynchronize(0), "set_values");
        cuda_check(cudaStreamSynchronize(fields.setup), "set_values");
    }

    template<typename TF>
    void Boundary<TF>::set_prognostic_cyclic_bcs(cudaStream_t s)
    {
        mhh_ctx* c = grid.ctx();
        for (auto* m : {&fields.mp, &fields.sp})
            for (auto& it : *m)
                check(mhh_boundary_cyclic(c, it.second->fld_g, MHH_EDGE_BOTH, s), "cyclic");
    }

    template<typename TF>
    void Boundary<TF>::set_ghost_cells(cudaStream_t s)
    {
        mhh_ctx* c = grid.ctx();
        for (const char* n : {"u", "v"})
        {
            auto& f = *fields.mp.at(n);
            check(mhh_boundary_ghost_cells(c, f.fld_g, mbcbot, f.fld_bot_g, f.grad_bot_g, mbctop, f.fld_top_g, f.grad_top_g, s), "ghost");
        }
        if (fields.sp.count("th"))
        {
            auto& f = *fields.sp.at("th");
            check(mhh_boundary_ghost_cells(c, f.fld_g, sbcbot, f.fld_bot_g, f.grad_bot_g, sbctop, f.fld_top_g, f.grad_top_g, s), "ghost");
        }
    }

    template<typename TF>
    void Boundary<TF>::exec(cudaStream_t s)
    {
        if (swboundary != "surface") return;
        mhh_fields f = fields.dev();
        mhh_bcfields b = fields.bc();
        check(mhh_boundary_surface_exec(grid.ctx(), &f, &b, fields.sp.count("th") ? sbcbot : MHH_BC_FLUX, s), "surface");
    }

    template<typename TF>
    Thermo_dry<TF>::Thermo_dry(Grid<TF>& g, Fields<TF>& f, Input& in) : grid(g), fields(f)
    {
        swthermo = in.get_item<std::string>("thermo", "swthermo", "", "0") == "dry";
    }

    template<typename TF>
    void Thermo_dry<TF>::exec(double, cudaStream_t s)
    {
        if (!swthermo) return;
        mhh_fields f = fields.dev();
        check(mhh_thermo_dry_exec(grid.ctx(), &f, s), "thermo");
    }

    template<typename TF>
    Force<TF>::Force(Grid<TF>& g, Fields<TF>& f, Input& in) : grid(g), fields(f)
    {
        const std::string sw = in.get_item<std::string>("force", "swlspres", "", "0");
        if (sw != "0" && sw != "dpdx") throw std::runtime_error("only swlspres=0 or dpdx is on this path");
        dpdx_on = sw == "dpdx";
        dpdx = dpdx_on ? in.get_item<double>("force", "dpdx", "") : 0.;
    }

    template<typename TF>
    void Force<TF>::exec(double, cudaStream_t s)
    {
        if (!dpdx_on) return;
        mhh_fields f = fields.dev();
        check(mhh_force_dpdx_exec(grid.ctx(), &f, dpdx, s), "force");
    }

    // ---------------------------------------------------------------------
    // Buffer, src/buffer.cxx:61-200
    // ---------------------------------------------------------------------
    template<typename TF>
    Buffer<TF>::Buffer(Grid<TF>& g, Fields<TF>& f, Input& in) : grid(g), fields(f)
    {
        swbuffer = in.get_item<bool>("buffer", "swbuffer", "", false);
        zstart = sigma = beta = 0.;
        if (swbuffer)
        {
            if (in.get_item<bool>("buffer", "swupdate", "", false))
                throw std::runtime_error("buffer swupdate=true is not on this path");
            zstart = in.get_item<double>("buffer", "zstart", "");
            sigma = in.get_item<double>("buffer", "sigma", "", 2.);
            beta = in.get_item<double>("buffer", "beta", "", 2.);
        }
    }

    template<typename TF>
    void Buffer<TF>::create()
    {
        if (swbuffer) check(mhh_buffer_setup(grid.ctx(), zstart, sigma, beta), "buffer setup");
    }

    template<typename TF>
    void Buffer<TF>::set_profile(const std::string& name, const double* prof)
    {
        if (!swbuffer) throw std::runtime_error("the buffer layer is off (swbuffer=false)");
        check(mhh_buffer_set_profile(grid.ctx(), name.c_str(), prof), "buffer profile");
    }

    template<typename TF>
    void Buffer<TF>::exec(cudaStream_t s)
    {
        if (!swbuffer) return;
        mhh_fields f = fields.dev();
        check(mhh_buffer_exec(grid.ctx(), &f, s), "buffer");
    }

    // ---------------------------------------------------------------------
    // Advec, src/advec.cxx:38-96 and the schemes.
    // ---------------------------------------------------------------------
    template<typename TF>
    Advec<TF>::Advec(Grid<TF>& g, Fields<TF>& f, Input& in) : grid(g), fields(f)
    {
        cflmax = in.get_item<double>("advec", "cflmax", "", 1.);
    }

    template<typename TF>
    std::unique_ptr<Advec<TF>> Advec<TF>::factory(Grid<TF>& g, Fields<TF>& f, Input& in)
    {
        const std::string sw = in.get_item<std::string>("advec", "swadvec", "", "2");
        if (sw == "2i5") return std::make_unique<Advec_2i5<TF>>(g, f, in);
        if (sw == "2") return std::make_unique<Advec_2<TF>>(g, f, in);
        throw std::runtime_error("swadvec = \"" + sw + "\" is not on this path (2 or 2i5)");
    }

    template<typename TF>
    double Advec<TF>::get_cfl(double dt)
    {
        mhh_fields f = fields.dev();
        double cfl;
        check(mhh_advec_get_cfl(grid.ctx(), get_switch(), &f, dt, &cfl, stream), "get_cfl");
        return cfl;
    }

    template<typename TF>
    unsigned long Advec<TF>::get_time_limit(unsigned long idt, double dt)
    {
        mhh_fields f = fields.dev();
        unsigned long long lim;
        check(mhh_advec_get_time_limit(grid.ctx(), get_switch(), &f, idt, dt, &lim, stream), "get_time_limit");
        return (unsigned long)lim;
    }

    template<typename TF>
    Advec_2i5<TF>::Advec_2i5(Grid<TF>& g, Fields<TF>& f, Input& in) : Advec<TF>(g, f, in)
    {
        const auto list = in.get_list("advec", "fluxlimit_list", "", {});
        for (const auto& n : list)
            if (n != "th") throw std::runtime_error("fluxlimit_list: only th is a scalar on this path");
        const bool lim = !list.empty() && f.sp.count("th");
        check(mhh_advec_2i5_set_fluxlimit(g.ctx(), lim ? 1 : 0), "fluxlimit");
    }

    template<typename TF>
    int Advec_2i5<TF>::kgc(Input& in)
    {
        // The limited scalar's stencil reaches two levels (src/advec_2i5.cxx:44).
        return in.get_list("advec", "fluxlimit_list", "", {}).empty() ? 1 : 2;
    }

    template<typename TF>
    void Advec_2i5<TF>::exec(Stats<TF>&)
    {
        mhh_fields f = this->fields.dev();
        check(mhh_advec_2i5_exec(this->grid.ctx(), &f, this->stream), "advec_2i5");
    }

    template<typename TF>
    void Advec_2<TF>::exec(Stats<TF>&)
    {
        mhh_fields f = this->fields.dev();
        check(mhh_advec_2_exec(this->grid.ctx(), &f, this->stream), "advec_2");
    }

    // ---------------------------------------------------------------------
    // Diff, src/diff.cxx:43-95 and the schemes.
    // ---------------------------------------------------------------------
    template<typename TF>
    Diff<TF>::Diff(Grid<TF>& g, Fields<TF>& f, Boundary<TF>& b, Input& in) : grid(g), fields(f), boundary(b)
    {
        dnmax = in.get_item<double>("diff", "dnmax", "", 0.4);
        tPr = TF(in.get_item<double>("diff", "tPr", "", 1./3.));
    }

    template<typename TF>
    std::unique_ptr<Diff<TF>> Diff<TF>::factory(Grid<TF>& g, Fields<TF>& f, Boundary<TF>& b, Input& in)
    {
        const std::string sw = in.get_item<std::string>("diff", "swdiff", "", "2");
        if (sw == "smag2") return std::make_unique<Diff_smag2<TF>>(g, f, b, in);
        if (sw == "2") return std::make_unique<Diff_2<TF>>(g, f, b, in);
        throw std::runtime_error("swdiff = \"" + sw + "\" is not on this path (2 or smag2)");
    }

    template<typename TF>
    Diff_smag2<TF>::Diff_smag2(Grid<TF>& g, Fields<TF>& f, Boundary<TF>& b, Input& in) : Diff<TF>(g, f, b, in) {}

    template<typename TF>
    void Diff_smag2<TF>::exec_viscosity(Stats<TF>&, Thermo_dry<TF>&)
    {
        mhh_fields f = this->fields.dev();
        mhh_bcfields b = this->fields.bc();
        check(mhh_diff_smag2_exec_viscosity(this->grid.ctx(), &f, &b, this->stream), "exec_viscosity");
    }

    template<typename TF>
    void Diff_smag2<TF>::exec(Stats<TF>&)
    {
        mhh_fields f = this->fields.dev();
        mhh_bcfields b = this->fields.bc();
        check(mhh_diff_smag2_exec(this->grid.ctx(), &f, &b, this->stream), "diff_smag2");
    }

    template<typename TF>
    double Diff_smag2<TF>::get_dn(double dt)
    {
        mhh_fields f = this->fields.dev();
        double dn;
        check(mhh_diff_smag2_get_dn(this->grid.ctx(), &f, dt, &dn, this->stream), "get_dn");
        return dn;
    }

    // src/diff_smag2.cxx:311-333
    template<typename TF>
    unsigned long Diff_smag2<TF>::get_time_limit(unsigned long idt, double dt)
    {
        double dnmul = get_dn(1.);
        dnmul = std::max(1.e-9, dnmul);
        return (unsigned long)((double)idt*this->dnmax/(dt*dnmul));
    }

    template<typename TF>
    void Diff_2<TF>::exec(Stats<TF>&)
    {
        mhh_fields f = this->fields.dev();
        check(mhh_diff_2_exec(this->grid.ctx(), &f, this->stream), "diff_2");
    }

    template<typename TF>
    double Diff_2<TF>::get_dn(double dt)
    {
        double dn;
        check(mhh_diff_2_get_dn(this->grid.ctx(), dt, &dn), "get_dn");
        return dn;
    }

    template<typename TF>
    unsigned long Diff_2<TF>::get_time_limit(unsigned long idt, double dt)
    {
        const double dnmul = get_dn(1.);
        return (unsigned long)((double)idt*this->dnmax/(dt*dnmul));
    }

    // ---------------------------------------------------------------------
    // Pres
    // ---------------------------------------------------------------------
    template<typename TF>
    Pres<TF>::Pres(Grid<TF>& g, Fields<TF>& f, Input& in) : grid(g), fields(f)
    {
        const std::string sw = in.get_item<std::string>("pres", "swpres", "", "2");
        if (sw != "2") throw std::runtime_error("only swpres=2 is on this path");
    }

    template<typename TF>
    std::unique_ptr<Pres<TF>> Pres<TF>::factory(Grid<TF>& g, Fields<TF>& f, Input& in)
    {
        return std::make_unique<Pres_2<TF>>(g, f, in);
    }

    template<typename TF>
    void Pres_2<TF>::exec(double dt, Stats<TF>&)
    {
        mhh_fields f = this->fields.dev();
        check(mhh_pres_2_exec(this->grid.ctx(), &f, dt, this->stream), "pres_2");
    }

    template<typename TF>
    TF Pres_2<TF>::check_divergence()
    {
        mhh_fields f = this->fields.dev();
        double div;
        check(mhh_pres_2_get_divergence(this->grid.ctx(), &f, &div, this->stream), "divergence");
        return TF(div);
    }

    // ---------------------------------------------------------------------
    // Timeloop, src/timeloop.cxx:42-176, :229-246, :358-423 (RK3)
    // ---------------------------------------------------------------------
    static unsigned long to_itime(double t) { return (unsigned long)(1e9*t + 0.5); }

    template<typename TF>
    Timeloop<TF>::Timeloop(Grid<TF>& g, Fields<TF>& f, Input& in) : grid(g), fields(f)
    {
        adaptivestep = in.get_item<bool>("time", "adaptivestep", "", true);
        dtmax = in.get_item<double>("time", "dtmax", "", 1.e9);
        dt = in.get_item<double>("time", "dt", "", dtmax);
        const int rk = in.get_item<int>("time", "rkorder", "", 3);
        if (rk != 3) throw std::runtime_error("only rkorder=3 is on this path");
        in.get_item<double>("time", "starttime", "", 0.);
        in.get_item<double>("time", "endtime", "", 0.);
        in.get_item<double>("time", "savetime", "", 0.);
        time = 0.; itime = 0; iteration = 0; substep = 0;
        idt = to_itime(dt); idtmax = to_itime(dtmax); idtlim = idt;
        const int iotimeprec = in.get_item<int>("time", "iotimeprec", "", 0);
        iiotimeprec = to_itime(std::pow(10., iotimeprec));
        outputiter = in.get_item<int>("time", "outputiter", "", 20);
        if (outputiter < 0) throw std::runtime_error("outputiter must be >= 0");
    }

    template<typename TF>
    void Timeloop<TF>::set_state(unsigned long itime_in, unsigned long idt_in, int iteration_in)
    {
        itime = itime_in; idt = idt_in; iteration = iteration_in;
        time = double(itime)/1e9;
        dt = double(idt)/1e9;
        substep = 0;
    }

    template<typename TF>
    void Timeloop<TF>::set_time_step()
    {
        if (in_substep()) return;
        if (adaptivestep)
        {
            if (idt == 0 || idtlim == 0)
                throw std::runtime_error("Required time step less than precision 1e-09 of the time stepping");
            idt = idtlim;
            dt = (double)idt / 1e9;
        }
    }

    template<typename TF>
    double Timeloop<TF>::get_sub_time_step() const
    {
        const double cB[3] = {1./3., 15./16., 8./15.};
        return cB[substep]*dt;
    }

    template<typename TF>
    void Timeloop<TF>::exec(cudaStream_t s)
    {
        mhh_ctx* c = grid.ctx();
        for (const char* n : {"u", "v", "w"})
            check(mhh_timeloop_rk3(c, fields.mp.at(n)->fld_g, fields.mt.at(n)->fld_g, substep, dt, s), "rk3");
        for (auto& it : fields.sp)
            check(mhh_timeloop_rk3(c, it.second->fld_g, fields.st.at(it.first)->fld_g, substep, dt, s), "rk3");
        advance_substep();
    }

    template<typename TF>
    void Timeloop<TF>::step_time()
    {
        if (in_substep()) return;
        time += dt;
        itime += idt;
        ++iteration;
    }

    // ---------------------------------------------------------------------
    // Model
    // ---------------------------------------------------------------------
    template<typename TF>
    Model<TF>::Model(const std::string& ini) : ini_text(ini)
    {
        input = std::make_unique<Input>(ini_text);
        const std::string swadvec = input->get_item<std::string>("advec", "swadvec", "", "2");
        grid = std::make_unique<Grid<TF>>(*input, swadvec == "2i5" ? 3 : 1,
                                          swadvec == "2i5" ? Advec_2i5<TF>::kgc(*input) : 1);
    }

    template<typename TF>
    void Model<TF>::init(const std::vector<double>& z)
    {
        z_full = z;
        grid->create(z);
        adaptive_ = input->get_item<bool>("time", "adaptivestep", "", true);
        const std::string swdiff = input->get_item<std::string>("diff", "swdiff", "", "2");
        fields = std::make_unique<Fields<TF>>(*grid, *input, grid->phys.thermo != 0, swdiff == "smag2");
        boundary = std::make_unique<Boundary<TF>>(*grid, *fields, *input);
        thermo = std::make_unique<Thermo_dry<TF>>(*grid, *fields, *input);
        force = std::make_unique<Force<TF>>(*grid, *fields, *input);
        buffer = std::make_unique<Buffer<TF>>(*grid, *fields, *input);
        buffer->create();
        advec = Advec<TF>::factory(*grid, *fields, *input);
        diff = Diff<TF>::factory(*grid, *fields, *boundary, *input);
        pres = Pres<TF>::factory(*grid, *fields, *input);
        timeloop = std::make_unique<Timeloop<TF>>(*grid, *fields, *input);
        boundary->set_values();
        std::memset(&cfg, 0, sizeof(cfg));
        cfg.advec = advec->get_switch();
        cfg.diff = diff->get_switch();
        cfg.swlspres = force->dpdx_on ? 1 : 0;
        cfg.dpdx = force->dpdx;
        cfg.mbcbot = boundary->mbcbot; cfg.mbctop = boundary->mbctop;
        cfg.sbcbot = boundary->sbcbot; cfg.sbctop = boundary->sbctop;
    }

    template<typename TF>
    Model<TF>::~Model()
    {
        cudaStreamSynchronize(stream);
        cudaStreamSynchronize(0);
        pres.reset(); diff.reset(); advec.reset(); buffer.reset(); force.reset(); thermo.reset(); boundary.reset();
        fields.reset(); timeloop.reset(); grid.reset();
    }

    template<typename TF>
    void Model<TF>::set_field(const std::string& name, const double* data) { fields->set_from_host(name, data); }

    template<typename TF>
    void Model<TF>::get_field(const std::string& name, double* data)
    {
        cuda_check(cudaStreamSynchronize(stream), "sync");
        fields->get_to_host(name, data);
    }

    template<typename TF>
    void Model<TF>::set_time_step()
    {
        // src/model.cxx:765-786
        if (timeloop->in_substep()) return;
        timeloop->set_time_step_limit();
        timeloop->set_time_step_limit(advec->get_time_limit(timeloop->get_idt(), timeloop->get_dt()));
        timeloop->set_time_step_limit(diff->get_time_limit(timeloop->get_idt(), timeloop->get_dt()));
        timeloop->set_time_step();
    }

    template<typename TF>
    void Model<TF>::substep_modules()
    {
        advec->set_stream(stream); diff->set_stream(stream); pres->set_stream(stream);
        // src/model.cxx:367-505
        boundary->set_prognostic_cyclic_bcs(stream);
        boundary->set_ghost_cells(stream);
        diff->exec_viscosity(stats, *thermo);
        set_time_step();
        thermo->exec(timeloop->get_sub_time_step(), stream);
        boundary->exec(stream);
        boundary->set_ghost_cells(stream);
        advec->exec(stats);
        diff->exec(stats);
        buffer->exec(stream);
        force->exec(timeloop->get_sub_time_step(), stream);
        pres->exec(timeloop->get_sub_time_step(), stats);
        timeloop->exec(stream);
        timeloop->step_time();
    }

    template<typename TF>
    void Model<TF>::substep_fused()
    {
        mhh_fields f = fields->dev();
        mhh_bcfields b = fields->bc();
        check(mhh_substep_begin(grid->ctx(), &cfg, &f, &b, stream), "substep_begin");
        // The limits only matter with an adaptive time step; with a fixed
        // step they would cost a synchronisation and change nothing.
        if (!timeloop->in_substep() && adaptive_)
            set_time_step();
        check(mhh_substep_end(grid->ctx(), &cfg, &f, &b, timeloop->get_substep(), timeloop->get_dt(), stream), "substep_end");
        timeloop->advance_substep();
        timeloop->step_time();
    }

    template<typename TF>
    void Model<TF>::substep_args(mhh_substep_config& c, mhh_fields& f, mhh_bcfields& b, double& dt) const
    {
        c = cfg;
        f = fields->dev();
        b = fields->bc();
        dt = timeloop->get_dt();
    }

    template<typename TF>
    void Model<TF>::advance_substep_host()
    {
        timeloop->advance_substep();
        timeloop->step_time();
    }

    template<typename TF>
    void Model<TF>::check_status()
    {
        if (!timeloop->do_check()) return;
        boundary->set_prognostic_cyclic_bcs(stream);
        mhh_fields f = fields->dev();
        double cfl = 0.;
        const int rc = mhh_advec_get_cfl(grid->ctx(), advec->get_switch(), &f, timeloop->get_dt(), &cfl, stream);
        if (rc == MHH_ERR_NONFINITE || (rc == MHH_OK && !(cfl >= 0. && cfl < 10.)))
            throw Nonfinite_error("Simulation has non-finite numbers");
        check(rc, "get_cfl");
    }

    template<typename TF>
    void Model<TF>::run_substeps(int n, bool fused)
    {
        for (int q=0; q<n; ++q)
        {
            check_status();
            if (fused) substep_fused();
            else substep_modules();
        }
    }

    template<typename TF>
    void Model<TF>::run_steps(int n, bool fused) { run_substeps(3*n, fused); }

    template<typename TF>
    void Model<TF>::set_buffer_profile(const std::string& name, const double* prof) { buffer->set_profile(name, prof); }

    template<typename TF>
    double Model<TF>::get_cfl()
    {
        boundary->set_prognostic_cyclic_bcs(stream);
        return advec->get_cfl(timeloop->get_dt());
    }

    template<typename TF>
    double Model<TF>::get_dn() { return diff->get_dn(timeloop->get_dt()); }

    template<typename TF>
    double Model<TF>::get_div()
    {
        boundary->set_prognostic_cyclic_bcs(stream);
        return double(pres->check_divergence());
    }

    template class Model<double>;
    template class Model<float>;

    namespace
    {
        std::string restart_name(const std::string& dir, const std::string& name, int iotime)
        {
            char buf[64];
            std::snprintf(buf, sizeof(buf), "%s.%07d", name.c_str(), iotime);
            return dir.empty() ? std::string(buf) : dir + "/" + buf;
        }

        // Exclusive create, as the reference's "wbx": a restart file is never
        // overwritten.
        FILE* create_exclusive(const std::string& path)
        {
            FILE* f = std::fopen(path.c_str(), "wbx");
            if (!f) throw std::runtime_error("cannot create " + path + " (exists or not writable)");
            return f;
        }

        template<typename T>
        void write_all(FILE* f, const T* p, size_t n, const std::string& path)
        {
            if (std::fwrite(p, sizeof(T), n, f) != n) { std::fclose(f); throw std::runtime_error("write error in " + path); }
        }

        template<typename T>
        void read_all(const std::string& path, T* p, size_t n)
        {
            FILE* f = std::fopen(path.c_str(), "rb");
            if (!f) throw std::runtime_error(path + " does not exist");
            const size_t got = std::fread(p, sizeof(T), n, f);
            std::fclose(f);
            if (got != n) throw std::runtime_error("short read in " + path);
        }
    }

    template<typename TF>
    int Model<TF>::save(const std::string& dir)
    {
        if (timeloop->in_substep()) throw std::runtime_error("save between full RK3 steps only");
        cuda_check(cudaStreamSynchronize(stream), "sync");
        const mhh_grid& g = grid->get_grid_data();
        const int iotime = timeloop->get_iotime();
        std::vector<double> full(g.ncells);
        // Prognostic 3-D fields: interior levels kstart..kend-1, rows of itot,
        // in the model precision.
        std::vector<std::string> names = {"u", "v", "w"};
        if (fields->sp.count("th")) names.push_back("th");
        for (const auto& n : names)
        {
            fields->get_to_host(n, full.data());
            {
                const std::string path = restart_name(dir, n, iotime);
                FILE* f = create_exclusive(path);
                std::vector<TF> row(g.itot);
                for (int k=g.kstart; k<g.kend; ++k)
                    for (int j=g.jstart; j<g.jend; ++j)
                    {
                        for (int i=0; i<g.itot; ++i) row[i] = TF(full[g.istart + i + (size_t)j*g.icells + (size_t)k*g.ijcells]);
                        write_all(f, row.data(), row.size(), path);
                    }
                std::fclose(f);
            }
            // The reference's file holds the physical field; a scalar stored
            // with an offset also gets <name>_stored.%07d with the stored
            // values as they are on the device (a physical value in double
            // cannot hold every bit of a small stored anomaly), so that a
            // restart continues bit for bit.
            if (fields->offset(n) != 0.)
            {
                std::vector<TF> raw(g.ncells);
                cuda_check(cudaMemcpy(raw.data(), fields->by_name(n)->fld_g, sizeof(TF)*g.ncells, cudaMemcpyDeviceToHost),
                           "copy");
                const std::string path = restart_name(dir, n + "_stored", iotime);
                FILE* f = create_exclusive(path);
                for (int k=g.kstart; k<g.kend; ++k)
                    for (int j=g.jstart; j<g.jend; ++j)
                        write_all(f, raw.data() + g.istart + (size_t)j*g.icells + (size_t)k*g.ijcells, (size_t)g.itot, path);
                std::fclose(f);
            }
        }
        // The integer time.
        {
            const std::string path = restart_name(dir, "time", iotime);
            FILE* f = create_exclusive(path);
            const unsigned long it = timeloop->get_itime(), idt = timeloop->get_idt();
            const int iter = timeloop->get_iteration();
            write_all(f, &it, 1, path);
            write_all(f, &idt, 1, path);
            write_all(f, &iter, 1, path);
            std::fclose(f);
        }
        // Surface model: the MO gradients of the last substep (the next
        // viscosity uses them) and the scalar's bottom gradient of a flux BC.
        if (boundary->get_switch() == "surface")
        {
            std::vector<double> a2(g.ijcells);
            std::vector<std::string> mo = {"dudz", "dvdz"};
            if (fields->sp.count("th")) mo.push_back("dbdz");
            for (const auto& n : mo)
            {
                check(mhh_boundary_surface_get(grid->ctx(), n.c_str(), a2.data()), "surface_get");
                const std::string path = restart_name(dir, n + "_mo", iotime);
                FILE* f = create_exclusive(path);
                std::vector<double> plane((size_t)g.itot*g.jtot);
                for (int j=0; j<g.jtot; ++j)
                    for (int i=0; i<g.itot; ++i)
                        plane[i + (size_t)j*g.itot] = a2[g.istart + i + (size_t)(j + g.jstart)*g.icells];
                write_all(f, plane.data(), plane.size(), path);
                std::fclose(f);
            }
            if (fields->sp.count("th") && boundary->sbcbot == MHH_BC_FLUX)
            {
                std::vector<TF> gb(g.ijcells);
                cuda_check(cudaMemcpy(gb.data(), fields->sp.at("th")->grad_bot_g, sizeof(TF)*g.ijcells,
                                      cudaMemcpyDeviceToHost), "copy");
                const std::string path = restart_name(dir, "th_gradbot", iotime);
                FILE* f = create_exclusive(path);
                std::vector<TF> plane((size_t)g.itot*g.jtot);
                for (int j=0; j<g.jtot; ++j)
                    for (int i=0; i<g.itot; ++i)
                        plane[i + (size_t)j*g.itot] = gb[g.istart + i + (size_t)(j + g.jstart)*g.icells];
                write_all(f, plane.data(), plane.size(), path);
                std::fclose(f);
            }
        }
        return iotime;
    }

    template<typename TF>
    void Model<TF>::load(const std::string& dir, int iotime)
    {
        cuda_check(cudaStreamSynchronize(stream), "sync");
        const mhh_grid& g = grid->get_grid_data();
        std::vector<std::string> names = {"u", "v", "w"};
        if (fields->sp.count("th")) names.push_back("th");
        const size_t nint = (size_t)g.itot*g.jtot*g.ktot;
        std::vector<TF> buf(nint);
        std::vector<double> full(g.ncells, 0.);
        for (const auto& n : names)
        {
            // The stored values where this implementation wrote them (exact),
            // else the reference's file of physical values.
            if (fields->offset(n) != 0.)
            {
                const std::string stored = restart_name(dir, n + "_stored", iotime);
                if (FILE* t = std::fopen(stored.c_str(), "rb"))
                {
                    std::fclose(t);
                    read_all(stored, buf.data(), nint);
                    std::vector<TF> raw(g.ncells, TF(0));
                    for (int k=0; k<g.ktot; ++k)
                        for (int j=0; j<g.jtot; ++j)
                            std::copy(buf.data() + (size_t)j*g.itot + (size_t)k*g.itot*g.jtot,
                                      buf.data() + (size_t)j*g.itot + (size_t)k*g.itot*g.jtot + g.itot,
                                      raw.data() + g.istart + (size_t)(j + g.jstart)*g.icells + (size_t)(k + g.kstart)*g.ijcells);
                    cuda_check(cudaMemcpy(fields->by_name(n)->fld_g, raw.data(), sizeof(TF)*g.ncells,
                                          cudaMemcpyHostToDevice), "copy");
                    continue;
                }
            }
            read_all(restart_name(dir, n, iotime), buf.data(), nint);
            std::fill(full.begin(), full.end(), 0.);
            for (int k=0; k<g.ktot; ++k)
                for (int j=0; j<g.jtot; ++j)
                    for (int i=0; i<g.itot; ++i)
                        full[g.istart + i + (size_t)(j + g.jstart)*g.icells + (size_t)(k + g.kstart)*g.ijcells]
                            = double(buf[i + (size_t)j*g.itot + (size_t)k*g.itot*g.jtot]);
            fields->set_from_host(n, full.data());
        }
        // The tendencies are zero between full steps.
        for (auto* m : {&fields->mt, &fields->st})
            for (auto& it : *m)
                cuda_check(cudaMemset(it.second->fld_g, 0, sizeof(TF)*g.ncells), "memset");
        {
            unsigned long it = 0, idt = 0;
            int iter = 0;
            const std::string path = restart_name(dir, "time", iotime);
            FILE* f = std::fopen(path.c_str(), "rb");
            if (!f) throw std::runtime_error(path + " does not exist");
            const bool ok = std::fread(&it, sizeof(it), 1, f) == 1 && std::fread(&idt, sizeof(idt), 1, f) == 1
                         && std::fread(&iter, sizeof(iter), 1, f) == 1;
            std::fclose(f);
            if (!ok) throw std::runtime_error("short read in " + path);
            timeloop->set_state(it, idt, iter);
        }
        if (boundary->get_switch() == "surface")
        {
            std::vector<double> plane((size_t)g.itot*g.jtot), a2(g.ijcells, 0.);
            std::vector<std::string> mo = {"dudz", "dvdz"};
            if (fields->sp.count("th")) mo.push_back("dbdz");
            for (const auto& n : mo)
            {
                read_all(restart_name(dir, n + "_mo", iotime), plane.data(), plane.size());
                // Interior plus the periodic ghost columns and rows.
                for (int j=0; j<g.jcells; ++j)
                    for (int i=0; i<g.icells; ++i)
                    {
                        const int ii = ((i - g.istart) % g.itot + g.itot) % g.itot;
                        const int jj = ((j - g.jstart) % g.jtot + g.jtot) % g.jtot;
                        a2[i + (size_t)j*g.icells] = plane[ii + (size_t)jj*g.itot];
                    }
                check(mhh_boundary_surface_set(grid->ctx(), n.c_str(), a2.data()), "surface_set");
            }
            if (fields->sp.count("th") && boundary->sbcbot == MHH_BC_FLUX)
            {
                std::vector<TF> p((size_t)g.itot*g.jtot), gb(g.ijcells);
                cuda_check(cudaMemcpy(gb.data(), fields->sp.at("th")->grad_bot_g, sizeof(TF)*g.ijcells,
                                      cudaMemcpyDeviceToHost), "copy");
                read_all(restart_name(dir, "th_gradbot", iotime), p.data(), p.size());
                for (int j=0; j<g.jcells; ++j)
                    for (int i=0; i<g.icells; ++i)
                    {
                        const int ii = ((i - g.istart) % g.itot + g.itot) % g.itot;
                        const int jj = ((j - g.jstart) % g.jtot + g.jtot) % g.jtot;
                        gb[i + (size_t)j*g.icells] = p[ii + (size_t)jj*g.itot];
                    }
                cuda_check(cudaMemcpy(fields->sp.at("th")->grad_bot_g, gb.data(), sizeof(TF)*g.ijcells,
                                      cudaMemcpyHostToDevice), "copy");
            }
        }
    }

    template int Model<double>::save(const std::string&);
    template int Model<float>::save(const std::string&);
    template void Model<double>::load(const std::string&, int);
    template void Model<float>::load(const std::string&, int);

    size_t estimate_model_bytes(const std::string& ini_text, int ktot, int precision)
    {
        Input in(ini_text);
        const std::string swadvec = in.get_item<std::string>("advec", "swadvec", "", "2");
        const int gc = swadvec == "2i5" ? 3 : 1;
        const int kgc = swadvec == "2i5" && !in.get_list("advec", "fluxlimit_list", "", {}).empty() ? 2 : 1;
        mhh_grid_desc d;
        d.itot = in.get_item<int>("grid", "itot", "");
        d.jtot = in.get_item<int>("grid", "jtot", "");
        d.ktot = ktot;
        d.igc = gc; d.jgc = gc; d.kgc = kgc;
        d.xsize = in.get_item<double>("grid", "xsize", "");
        d.ysize = in.get_item<double>("grid", "ysize", "");
        d.zsize = in.get_item<double>("grid", "zsize", "");
        size_t ctx = 0;
        check(mhh_ctx_estimate_bytes(&d, precision, &ctx), "estimate");
        const double tf = precision == MHH_FP64 ? 8. : 4.;
        const double ij = double(d.itot + 2*gc)*(d.jtot + 2*gc);
        const double nc = ij*(d.ktot + 2*kgc);
        // u v w th, their tendencies, p, evisc; 18 boundary arrays.
        return ctx + size_t(10.*nc*tf + 18.*ij*tf + 20.*2.*1024*1024);
    }
}

// ---------------------------------------------------------------------------
// C entry points (include/mhh_model.h)
// ---------------------------------------------------------------------------
namespace
{
    thread_local std::string g_model_error;

    using Handle = mhh_host::ModelHandle;

    template<typename F>
    int guard(F&& f)
    {
        try { f(); return MHH_OK; }
        catch (mhh_host::Nonfinite_error& e) { g_model_error = e.what(); return MHH_ERR_NONFINITE; }
        catch (std::exception& e) { g_model_error = e.what(); return MHH_ERR_ARG; }
    }
}

extern "C" {

const char* mhh_model_last_error(void) { return g_model_error.c_str(); }

int mhh_model_create(const char* ini_text, const double* z, int ktot, int precision, mhh_model** out)
{
    if (!ini_text || !z || !out) { g_model_error = "NULL argument"; return MHH_ERR_ARG; }
    auto* h = new Handle();
    h->prec = precision;
    const int rc = guard([&]
    {
        std::vector<double> zv(z, z + ktot);
        if (precision == MHH_FP64)
        {
            h->m64 = std::make_unique<mhh_host::Model<double>>(ini_text);
            h->m64->init(zv);
        }
        else if (precision == MHH_FP32)
        {
            h->m32 = std::make_unique<mhh_host::Model<float>>(ini_text);
            h->m32->init(zv);
        }
        else throw std::runtime_error("precision must be 64 or 32");
    });
    if (rc) { delete h; return rc; }
    *out = reinterpret_cast<mhh_model*>(h);
    return MHH_OK;
}

int mhh_model_destroy(mhh_model* mm)
{
    delete reinterpret_cast<Handle*>(mm);
    return MHH_OK;
}

#define WITH_MODEL(mm, body) \
    do { Handle* h_ = reinterpret_cast<Handle*>(mm); if (!h_) { g_model_error = "NULL model"; return MHH_ERR_ARG; } \
         return guard([&] { if (h_->prec == MHH_FP64) { auto& m = *h_->m64; body; } else { auto& m = *h_->m32; body; } }); } while (0)

int mhh_model_set_field(mhh_model* mm, const char* name, const double* data) { WITH_MODEL(mm, m.set_field(name, data)); }
int mhh_model_get_field(mhh_model* mm, const char* name, double* data) { WITH_MODEL(mm, m.get_field(name, data)); }
int mhh_model_set_field_native(mhh_model* mm, const char* name, const void* data)
{ WITH_MODEL(mm, m.get_fields().set_native(name, data, m.stream)); }
int mhh_model_get_field_native(mhh_model* mm, const char* name, void* data)
{ WITH_MODEL(mm, m.get_fields().get_native(name, data, m.stream)); }
int mhh_model_run_steps(mhh_model* mm, int n, int fused) { WITH_MODEL(mm, m.run_steps(n, fused != 0)); }
int mhh_model_run_substeps(mhh_model* mm, int n, int fused) { WITH_MODEL(mm, m.run_substeps(n, fused != 0)); }
int mhh_model_get_cfl(mhh_model* mm, double* out) { WITH_MODEL(mm, *out = m.get_cfl()); }
int mhh_model_get_dn(mhh_model* mm, double* out) { WITH_MODEL(mm, *out = m.get_dn()); }
int mhh_model_get_div(mhh_model* mm, double* out) { WITH_MODEL(mm, *out = m.get_div()); }
int mhh_model_get_dt(mhh_model* mm, double* out) { WITH_MODEL(mm, *out = m.get_timeloop().get_dt()); }
int mhh_model_get_time(mhh_model* mm, double* out) { WITH_MODEL(mm, *out = m.get_timeloop().get_time()); }
int mhh_model_get_substep(mhh_model* mm, int* out) { WITH_MODEL(mm, *out = m.get_timeloop().get_substep()); }
int mhh_model_get_grid(mhh_model* mm, mhh_grid* out) { WITH_MODEL(mm, *out = m.get_grid().get_grid_data()); }
int mhh_model_get_profile(mhh_model* mm, const char* name, double* out)
{ WITH_MODEL(mm, { auto v = m.get_grid().profile(name); std::copy(v.begin(), v.end(), out); }); }
int mhh_model_get_surface(mhh_model* mm, const char* name, double* out)
{ WITH_MODEL(mm, { mhh_host::cuda_check(cudaStreamSynchronize(m.stream), "sync");
                   mhh_host::check(mhh_boundary_surface_get(m.get_grid().ctx(), name, out), "surface_get"); }); }
int mhh_model_set_stream(mhh_model* mm, cudaStream_t s) { WITH_MODEL(mm, m.stream = s); }
int mhh_model_set_buffer_profile(mhh_model* mm, const char* name, const double* prof)
{
    if (!name || !prof) return MHH_ERR_ARG;
    WITH_MODEL(mm, m.set_buffer_profile(name, prof));
}
int mhh_model_synchronize(mhh_model* mm)
{ WITH_MODEL(mm, { cudaError_t e = cudaStreamSynchronize(m.stream); if (e != cudaSuccess) throw std::runtime_error(cudaGetErrorString(e)); }); }
int mhh_model_get_device_fields(mhh_model* mm, mhh_fields* f, mhh_bcfields* bc)
{ WITH_MODEL(mm, { *f = m.get_fields().dev(); *bc = m.get_fields().bc(); }); }
int mhh_model_save(mhh_model* mm, const char* dir, int* iotime)
{ WITH_MODEL(mm, { const int t = m.save(dir ? dir : ""); if (iotime) *iotime = t; }); }
int mhh_model_load(mhh_model* mm, const char* dir, int iotime) { WITH_MODEL(mm, m.load(dir ? dir : "", iotime)); }
mhh_ctx* mhh_model_get_ctx(mhh_model* mm)
{
    Handle* h = reinterpret_cast<Handle*>(mm);
    if (!h) return nullptr;
    return h->prec == MHH_FP64 ? h->m64->get_grid().ctx() : h->m32->get_grid().ctx();
}

}
