// ref_driver.cxx -- the oracle C API (mhh_oracle.h) on top of the reference's
// own module classes (TEST INFRASTRUCTURE ONLY).  The substep follows the
// run-mode loop of src/model.cxx:356-505; the modules are the reference's
// Advec_2i5 / Advec_2, Diff_smag2 / Diff_2, Pres_2, Timeloop, Boundary_cyclic,
// Boundary_surface and Buffer compiled unchanged.
#include <cstring>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "ref_harness.h"
#include "../mhh_oracle.h"
#include "../orc_fft.h"

#include "advec_2i5.h"
#include "advec_2.h"
#include "diff_smag2.h"
#include "diff_2.h"
#include "pres_2.h"
#include "fft.h"
#include "timeloop.h"
#include "boundary_surface.h"
#include "buffer.h"
#include "stats.h"
#include "constants.h"

using TF = double;

struct orc_model
{
    orc_params p;
    Master master;
    std::unique_ptr<Input> input;
    std::unique_ptr<Grid<TF>> grid;
    std::unique_ptr<Soil_grid<TF>> soil_grid;
    std::unique_ptr<Fields<TF>> fields;
    std::unique_ptr<Timeloop<TF>> timeloop;
    std::unique_ptr<FFT<TF>> fft;
    std::unique_ptr<Boundary<TF>> boundary;
    std::unique_ptr<ref_harness::Thermo_dry_ref> thermo;
    std::unique_ptr<Advec<TF>> advec;
    std::unique_ptr<Diff<TF>> diff;
    std::unique_ptr<Pres<TF>> pres;
    std::unique_ptr<Buffer<TF>> buffer;
    // The statistics object is never touched by the hot path (all its calls
    // are no-ops in the harness); it only has to exist as a reference.
    alignas(64) unsigned char stats_mem[sizeof(Stats<TF>)];
    alignas(64) unsigned char misc_mem[256];
    Stats<TF>& stats() { return *reinterpret_cast<Stats<TF>*>(stats_mem); }
};

namespace
{
    const char* bc_m(int t) { return t == ORC_BC_DIRICHLET ? "noslip" : "freeslip"; }
    const char* bc_s(int t) { return t == ORC_BC_DIRICHLET ? "dirichlet" : (t == ORC_BC_NEUMANN ? "neumann" : "flux"); }

    std::string make_input(const orc_params* p)
    {
        std::ostringstream s;
        s.precision(17);
        s << "grid itot - " << p->itot << "\n" << "grid jtot - " << p->jtot << "\n" << "grid ktot - " << p->ktot << "\n";
        s << "grid xsize - " << p->xsize << "\n" << "grid ysize - " << p->ysize << "\n" << "grid zsize - " << p->zsize << "\n";
        s << "grid swspatialorder - 2\n";
        s << "fields visc - " << p->visc << "\n" << "fields svisc - " << p->svisc << "\n";
        s << "advec swadvec - " << (p->advec == ORC_ADVEC_2I5 ? "2i5" : "2") << "\n";
        s << "advec cflmax - " << p->cflmax << "\n";
        if (p->fluxlimit_s) s << "advec fluxlimit_list - th\n";
        s << "diff swdiff - " << (p->diff == ORC_DIFF_SMAG2 ? "smag2" : "2") << "\n";
        s << "diff cs - " << p->cs << "\n" << "diff tPr - " << p->tpr << "\n" << "diff dnmax - " << p->dnmax << "\n";
        s << "diff swmason - " << (p->swmason ? 1 : 0) << "\n";
        s << "thermo thref0 - " << p->thref0 << "\n";
        s << "boundary mbcbot - " << bc_m(p->mbcbot) << "\n" << "boundary mbctop - " << bc_m(p->mbctop) << "\n";
        s << "boundary ubot - " << p->ubot << "\n" << "boundary utop - " << p->utop << "\n";
        s << "boundary vbot - " << p->vbot << "\n" << "boundary vtop - " << p->vtop << "\n";
        s << "boundary sbcbot th " << bc_s(p->sbcbot) << "\n" << "boundary sbctop th " << bc_s(p->sbctop) << "\n";
        s << "boundary sbot th " << p->sbot << "\n" << "boundary stop th " << p->stop << "\n";
        s << "boundary z0m - " << p->z0m << "\n" << "boundary z0h - " << p->z0h << "\n";
        s << "time starttime - 0\n" << "time endtime - 1e12\n" << "time savetime - 1e9\n";
        s << "time dt - " << p->dt << "\n";
        if (p->dtmax > 0.) s << "time dtmax - " << p->dtmax << "\n";
        s << "time adaptivestep - " << (p->adaptivestep ? 1 : 0) << "\n";
        s << "buffer swbuffer - " << (p->swbuffer ? 1 : 0) << "\n";
        if (p->swbuffer)
            s << "buffer zstart - " << p->buf_zstart << "\n" << "buffer sigma - " << p->buf_sigma << "\n"
              << "buffer beta - " << p->buf_beta << "\n";
        return s.str();
    }

    // src/force.cxx:626-636
    void exec_force(orc_model* m)
    {
        if (m->p.swlspres != 1) return;
        auto& gd = m->grid->get_grid_data();
        const TF fbody = TF(-1.)*m->p.dpdx;
        TF* ut = m->fields->mt.at("u")->fld.data();
        for (int k=gd.kstart; k<gd.kend; ++k)
            for (int j=gd.jstart; j<gd.jend; ++j)
                for (int i=gd.istart; i<gd.iend; ++i)
                    ut[i + j*gd.icells + k*gd.ijcells] += fbody;
    }

    // src/model.cxx:765-786
    void set_time_step(orc_model* m)
    {
        auto& tl = *m->timeloop;
        if (tl.in_substep()) return;
        tl.set_time_step_limit();
        tl.set_time_step_limit(m->advec->get_time_limit(tl.get_idt(), tl.get_dt()));
        tl.set_time_step_limit(m->diff->get_time_limit(tl.get_idt(), tl.get_dt()));
        tl.set_time_step();
    }

    Field3d<TF>* field_by_name(const orc_model* m, const std::string& n)
    {
        auto& f = *m->fields;
        if (n == "u" || n == "v" || n == "w") return f.mp.at(n).get();
        if (n == "ut" || n == "vt" || n == "wt") return f.mt.at(n.substr(0, 1)).get();
        if (n == "th") return f.sp.count("th") ? f.sp.at("th").get() : nullptr;
        if (n == "tht") return f.st.count("th") ? f.st.at("th").get() : nullptr;
        if (n == "p") return f.sd.at("p").get();
        if (n == "evisc") return f.sd.count("evisc") ? f.sd.at("evisc").get() : nullptr;
        return nullptr;
    }
}

extern "C" {

orc_model* orc_create(const orc_params* p, const double* z)
{
    auto* m = new orc_model();
    m->p = *p;
    m->master.start();
    m->input = std::make_unique<Input>(m->master, make_input(p));
    m->master.init(*m->input);
    auto& input = *m->input;

    m->grid = std::make_unique<Grid<TF>>(m->master, input);
    m->soil_grid = std::make_unique<Soil_grid<TF>>(m->master, *m->grid, input);
    m->fields = std::make_unique<Fields<TF>>(m->master, *m->grid, *m->soil_grid, input);
    m->fft = std::make_unique<FFT<TF>>(m->master, *m->grid);
    if (p->surface)
        m->boundary = std::make_unique<Boundary_surface<TF>>(m->master, *m->grid, *m->soil_grid, *m->fields, input);
    else
        m->boundary = std::make_unique<Boundary<TF>>(m->master, *m->grid, *m->soil_grid, *m->fields, input);

    // Modules in the order of src/model.cxx:109-167.
    if (p->advec == ORC_ADVEC_2I5)
        m->advec = std::make_unique<Advec_2i5<TF>>(m->master, *m->grid, *m->fields, input);
    else
        m->advec = std::make_unique<Advec_2<TF>>(m->master, *m->grid, *m->fields, input);
    if (p->diff == ORC_DIFF_SMAG2)
        m->diff = std::make_unique<Diff_smag2<TF>>(m->master, *m->grid, *m->fields, *m->boundary, input);
    else
        m->diff = std::make_unique<Diff_2<TF>>(m->master, *m->grid, *m->fields, *m->boundary, input);
    m->pres = std::make_unique<Pres_2<TF>>(m->master, *m->grid, *m->fields, *m->fft, input);
    m->buffer = std::make_unique<Buffer<TF>>(m->master, *m->grid, *m->fields, input);

    // Grid and fields (ghost-cell counts are final now).
    m->grid->init();
    ref_harness::set_pending_z(std::vector<double>(z, z + p->ktot));
    m->grid->create(input, *reinterpret_cast<Netcdf_handle*>(m->misc_mem));
    auto& gd = m->grid->get_grid_data();

    auto& f = *m->fields;
    f.init_momentum_field("u", "", "", "default", gd.uloc);
    f.init_momentum_field("v", "", "", "default", gd.vloc);
    f.init_momentum_field("w", "", "", "default", gd.wloc);
    if (p->thermo)
    {
        f.init_prognostic_field("th", "", "", "default", gd.sloc);
        f.sp.at("th")->visc = p->svisc;
    }
    f.init_diagnostic_field("p", "", "", "default", gd.sloc);
    for (auto& it : f.sd) it.second->init();
    f.rhoref.assign(gd.kcells, 1.);
    f.rhorefh.assign(gd.kcells, 1.);

    m->thermo = std::make_unique<ref_harness::Thermo_dry_ref>(m->master, *m->grid, *m->fields, input, p->thermo != 0);
    m->timeloop = std::make_unique<Timeloop<TF>>(m->master, *m->grid, *m->soil_grid, *m->fields, input, Sim_mode::Run);

    // Model::init and Model::load_or_save (src/model.cxx:185-300).
    m->boundary->init(input, *m->thermo, Sim_mode::Run);
    m->buffer->init();
    m->diff->init();
    m->pres->init();
    m->boundary->set_values();
    m->pres->set_values();
    m->advec->create(m->stats());
    m->diff->create(m->stats(), false);
    return m;
}

void orc_destroy(orc_model* m) { delete m; }

long orc_ncells(const orc_model* m) { return m->grid->get_grid_data().ncells; }

void orc_dims(const orc_model* m, int* d)
{
    auto& gd = m->grid->get_grid_data();
    d[0] = gd.igc; d[1] = gd.jgc; d[2] = gd.kgc; d[3] = gd.icells; d[4] = gd.jcells; d[5] = gd.kcells;
}

int orc_set_field(orc_model* m, const char* name, const double* data)
{
    Field3d<TF>* f = field_by_name(m, name);
    if (!f) return -1;
    std::memcpy(f->fld.data(), data, sizeof(double)*f->fld.size());
    return 0;
}

int orc_get_field(const orc_model* m, const char* name, double* data)
{
    Field3d<TF>* f = field_by_name(m, name);
    if (!f) return -1;
    std::memcpy(data, f->fld.data(), sizeof(double)*f->fld.size());
    return 0;
}

int orc_get_profile(const orc_model* m, const char* name, double* data)
{
    auto& gd = m->grid->get_grid_data();
    const std::string n(name);
    const std::vector<double>* v = nullptr;
    if (n == "z") v = &gd.z;
    else if (n == "zh") v = &gd.zh;
    else if (n == "dz") v = &gd.dz;
    else if (n == "dzh") v = &gd.dzh;
    else if (n == "dzi") v = &gd.dzi;
    else if (n == "dzhi") v = &gd.dzhi;
    else if (n == "rhoref") v = &m->fields->rhoref;
    else if (n == "rhorefh") v = &m->fields->rhorefh;
    if (!v) return -1;
    std::memcpy(data, v->data(), sizeof(double)*gd.kcells);
    return 0;
}

int orc_get_2d(const orc_model* m, const char* name, double* data)
{
    auto& gd = m->grid->get_grid_data();
    const std::string n(name);
    const std::vector<double>* v = nullptr;
    auto& f = *m->fields;
    if (n == "u_fluxbot") v = &f.mp.at("u")->flux_bot;
    else if (n == "v_fluxbot") v = &f.mp.at("v")->flux_bot;
    else if (n == "u_gradbot") v = &f.mp.at("u")->grad_bot;
    else if (n == "v_gradbot") v = &f.mp.at("v")->grad_bot;
    else if (n == "th_fluxbot" && f.sp.count("th")) v = &f.sp.at("th")->flux_bot;
    else if (n == "th_gradbot" && f.sp.count("th")) v = &f.sp.at("th")->grad_bot;
    else if (m->p.surface && (n == "dudz" || n == "dvdz" || n == "dbdz"))
    {
        if (n == "dudz") v = &m->boundary->get_dudz();
        else if (n == "dvdz") v = &m->boundary->get_dvdz();
        else if (m->p.thermo) v = &m->boundary->get_dbdz();
    }
    if (!v) return -1;
    std::memcpy(data, v->data(), sizeof(double)*gd.ijcells);
    return 0;
}

void orc_set_cyclic_and_ghost(orc_model* m)
{
    m->boundary->set_prognostic_cyclic_bcs();
    m->boundary->set_ghost_cells();
}

void orc_exec_viscosity(orc_model* m) { m->diff->exec_viscosity(m->stats(), *m->thermo); }
void orc_exec_thermo(orc_model* m) { m->thermo->exec(m->timeloop->get_sub_time_step(), m->stats()); }
void orc_exec_boundary(orc_model* m)
{
    m->boundary->exec(*m->thermo, *reinterpret_cast<Radiation<TF>*>(m->misc_mem),
                      *reinterpret_cast<Microphys<TF>*>(m->misc_mem), *m->timeloop);
}
void orc_exec_advec(orc_model* m) { m->advec->exec(m->stats()); }
void orc_exec_diff(orc_model* m) { m->diff->exec(m->stats()); }
void orc_exec_force(orc_model* m) { exec_force(m); }
void orc_exec_buffer(orc_model* m) { m->buffer->exec(m->stats()); }

// Buffer::create (src/buffer.cxx:100-158) reads the initial profiles; it runs
// again after every profile handed over, with the profiles given so far.
int orc_set_buffer_profile(orc_model* m, const char* name, const double* prof)
{
    const std::string n(name);
    if (!m->p.swbuffer || (n != "u" && n != "v" && n != "th")) return -1;
    auto& gd = m->grid->get_grid_data();
    ref_harness::set_init_profile(n, std::vector<double>(prof + gd.kstart, prof + gd.kend));
    m->buffer->create(*m->input, *reinterpret_cast<Netcdf_handle*>(m->misc_mem), m->stats());
    return 0;
}
void orc_exec_pres(orc_model* m, double sub_dt) { m->pres->exec(sub_dt, m->stats()); }
void orc_exec_timeloop(orc_model* m) { m->timeloop->exec(); m->timeloop->step_time(); }

void orc_run_substeps(orc_model* m, int n)
{
    for (int s=0; s<n; ++s)
    {
        orc_set_cyclic_and_ghost(m);
        orc_exec_viscosity(m);
        set_time_step(m);
        orc_exec_thermo(m);
        orc_exec_boundary(m);
        m->boundary->set_ghost_cells();
        orc_exec_advec(m);
        orc_exec_diff(m);
        orc_exec_buffer(m);
        orc_exec_force(m);
        orc_exec_pres(m, m->timeloop->get_sub_time_step());
        orc_exec_timeloop(m);
    }
}

double orc_get_cfl(orc_model* m) { return m->advec->get_cfl(m->timeloop->get_dt()); }
double orc_get_dn(orc_model* m) { return m->diff->get_dn(m->timeloop->get_dt()); }
double orc_get_div(orc_model* m) { return m->pres->check_divergence(); }
double orc_get_dt(const orc_model* m) { return m->timeloop->get_dt(); }
int orc_get_substep(const orc_model* m) { return m->timeloop->get_substep(); }
unsigned long orc_get_itime(const orc_model* m) { return m->timeloop->get_itime(); }

void orc_r2hc(int n, int howmany, double* data, long stride, long dist) { orcfft_r2hc(n, howmany, data, stride, dist); }
void orc_hc2r(int n, int howmany, double* data, long stride, long dist) { orcfft_hc2r(n, howmany, data, stride, dist); }
int orc_num_threads(void) { return 1; }

}
