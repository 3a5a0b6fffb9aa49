// ref_harness.h -- stub host layer that lets the reference's own hot-path
// sources (compiled unchanged from the MicroHH tree) run as a library
// (TEST INFRASTRUCTURE ONLY).
//
// The reference classes Advec_2i5, Advec_2, Diff_smag2, Diff_2, Pres_2,
// Timeloop, Boundary_cyclic and Boundary_surface are used as they are; this
// layer supplies what their .cxx files leave undefined: Input (from a string
// of "group key subkey value" lines instead of an .ini file), Grid (the
// 2nd-order metrics of src/grid.cxx:245-305), Fields storage, a dry
// Boussinesq thermodynamics (src/thermo_dry.cxx:64-181), the Boundary base
// class (src/boundary.cxx:156-1023) and an FFT (halfcomplex, on top of the
// oracle's orc_fft.c in place of FFTW).
#ifndef MHH_REF_HARNESS_H
#define MHH_REF_HARNESS_H

#include <string>
#include <vector>

#include "master.h"
#include "input.h"
#include "grid.h"
#include "soil_grid.h"
#include "fields.h"
#include "thermo.h"
#include "boundary.h"

namespace ref_harness
{
    // Heights of the ktot full levels handed to Grid<double>::create.
    void set_pending_z(const std::vector<double>& z);

    // Initial profiles (ktot interior values by name) that the stand-in
    // Netcdf_handle::get_variable returns to Buffer::create; a name without
    // an entry reads as zeros, as a missing variable does in
    // src/netcdf_interface.cxx:659-684.
    void set_init_profile(const std::string& name, const std::vector<double>& prof);

    // Dry Boussinesq thermodynamics with prognostic "th" (restated from
    // src/thermo_dry.cxx; only what the hot path calls).
    class Thermo_dry_ref : public Thermo<double>
    {
        public:
            Thermo_dry_ref(Master&, Grid<double>&, Fields<double>&, Input&, bool enabled);
            ~Thermo_dry_ref();

            void init() override {}
            void create(Input&, Netcdf_handle&, Stats<double>&, Column<double>&, Cross<double>&,
                        Dump<double>&, Timeloop<double>&) override {}
            void create_basestate(Input&, Netcdf_handle&, Timeloop<double>&) override {}
            unsigned long get_time_limit(unsigned long, double) override;
            void load(const int) override {}
            void save(const int) override {}
            void create_stats(Stats<double>&) override {}
            void exec(const double, Stats<double>&) override;
            void exec_stats(Stats<double>&) override {}
            void exec_column(Column<double>&) override {}
            void exec_dump(Dump<double>&, unsigned long) override {}
            void exec_cross(Cross<double>&, unsigned long) override {}
            void get_mask(Stats<double>&, std::string) override {}
            bool has_mask(std::string) override { return false; }
            bool check_field_exists(std::string name) override { return name == "N2"; }
            void get_thermo_field(Field3d<double>&, const std::string&, const bool, const bool) override;
            void get_buoyancy_surf(std::vector<double>&, std::vector<double>&, bool) override;
            void get_buoyancy_surf(std::vector<double>&, std::vector<double>&, std::vector<double>&) override;
            void get_buoyancy_fluxbot(std::vector<double>&, bool) override;
            void get_temperature_bot(Field3d<double>&, bool) override;
            void get_prog_vars(std::vector<std::string>&) override;
            void get_radiation_fields(Field3d<double>&, Field3d<double>&, Field3d<double>&,
                                      Field3d<double>&, Field3d<double>&) const override;
            void get_radiation_fields(Field3d<double>&, Field3d<double>&, Field3d<double>&,
                                      Field3d<double>&, Field3d<double>&, Field3d<double>&) const override;
            void get_radiation_columns(Field3d<double>&, std::vector<int>&, std::vector<int>&) const override;
            void get_land_surface_fields(std::vector<double>&, std::vector<double>&, std::vector<double>&,
                                         std::vector<double>&, std::vector<double>&) override;
            const std::vector<double>& get_basestate_vector(std::string) const override;
            double get_db_ref() const override;
            int get_bl_depth() override { return 0; }
            double get_buoyancy_diffusivity() override { return 0.; }
            void update_time_dependent(Timeloop<double>&) override {}

            std::vector<double> thref, threfh;
    };
}
#endif
