// mhh_host.h -- C++ host layer with the reference's class API for the
// LES/DNS time step (Input, Grid, Fields, Boundary, Thermo_dry, Force, Advec,
// Diff, Pres, Timeloop, Model), device-resident, on top of the C-ABI of
// include/mhh.h.  Class and member names follow the reference
// (include/advec.h:45-70, include/diff.h:37-71, include/pres.h:39-85,
// include/timeloop.h:49-139, src/model.cxx) so that a caller of those classes
// finds the same entry points; the arithmetic runs in the CUDA kernels behind
// the C-ABI.  Errors raise std::runtime_error, as in the reference.
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "mhh.h"

namespace mhh_host
{
    // ---- .ini input, src/input.cxx:77-222 -------------------------------
    class Input
    {
        public:
            explicit Input(const std::string& ini_text);
            template<typename T> T get_item(const std::string& group, const std::string& key, const std::string& sub);
            template<typename T> T get_item(const std::string& group, const std::string& key, const std::string& sub, const T def);
            // Comma-separated list of strings, src/input.cxx:224-263.
            std::vector<std::string> get_list(const std::string& group, const std::string& key, const std::string& sub,
                                              const std::vector<std::string>& def);
            std::vector<std::string> unused_items() const;
        private:
            bool find(const std::string& g, const std::string& k, const std::string& s, std::string& out);
            // group -> key -> subkey -> (value, used)
            std::map<std::string, std::map<std::string, std::map<std::string, std::pair<std::string, bool>>>> items;
    };

    void check(int rc, const char* what);

    // A run that has produced non-finite numbers (a reduction returned NaN or
    // inf, or the status check found the CFL number out of range).  The C
    // entry points return MHH_ERR_NONFINITE for it.
    struct Nonfinite_error : std::runtime_error
    {
        using std::runtime_error::runtime_error;
    };

    template<typename TF> class Grid;
    template<typename TF> class Fields;

    // Statistics are out of scope; the hooks the modules call are kept.
    template<typename TF> struct Stats { void calc_tend(const std::string&, const std::string&) {} };

    // ---- Grid, src/grid.cxx ----------------------------------------------
    template<typename TF>
    class Grid
    {
        public:
            Grid(Input&, int igc, int kgc);
            ~Grid();
            void create(const std::vector<double>& z);
            const mhh_grid& get_grid_data() const { return gd; }
            mhh_ctx* ctx() const { return ctx_; }
            std::vector<double> profile(const std::string& name) const;
            mhh_grid_desc desc;
            mhh_physics phys;
        private:
            mhh_grid gd;
            mhh_ctx* ctx_ = nullptr;
    };

    // ---- Field3d / Fields, include/field3d.h, include/fields.h ----------
    template<typename TF>
    struct Field3d
    {
        std::string name;
        TF* fld_g = nullptr;
        TF *fld_bot_g = nullptr, *fld_top_g = nullptr;
        TF *grad_bot_g = nullptr, *grad_top_g = nullptr;
        TF *flux_bot_g = nullptr, *flux_top_g = nullptr;
        double visc = 0.;
        cudaStream_t alloc_stream = nullptr;   // stream of the stream-ordered allocation and release
        Field3d(const std::string& n, long long ncells, int ijcells, cudaStream_t s);
        ~Field3d();
    };

    template<typename TF>
    class Fields
    {
        public:
            Fields(Grid<TF>&, Input&, bool with_scalar, bool with_evisc);
            ~Fields();
            cudaStream_t setup = nullptr;   // allocation and release stream of the fields
            std::map<std::string, std::shared_ptr<Field3d<TF>>> mp, mt, sp, st, sd;
            double visc, svisc;
            mhh_fields dev() const;          // device pointers for the C-ABI
            // Storage offset of field `name` (theta in FP32 contexts), else 0.
            double offset(const std::string& name) const;
            mhh_bcfields bc() const;
            // Host copies are physical values; the scalar th is stored on the
            // device with the context's offset (mhh_ctx_scalar_offset), which
            // these conversions add or remove.
            void set_from_host(const std::string& name, const double* data);
            void get_to_host(const std::string& name, double* data) const;
            // Host buffers already in the model precision (TF), copied on the
            // given stream (asynchronous for page-locked buffers).
            void set_native(const std::string& name, const void* data, cudaStream_t s);
            void get_native(const std::string& name, void* data, cudaStream_t s) const;
            Field3d<TF>* by_name(const std::string& name) const;
        private:
            Grid<TF>& grid;
    };

    // ---- Boundary, src/boundary.cxx + src/boundary_surface.cxx -----------
    template<typename TF>
    class Boundary
    {
        public:
            Boundary(Grid<TF>&, Fields<TF>&, Input&);
            void set_values();
            void set_prognostic_cyclic_bcs(cudaStream_t);
            void set_ghost_cells(cudaStream_t);
            void exec(cudaStream_t);                 // surface layer when swboundary=surface
            std::string get_switch() const { return swboundary; }
            int mbcbot, mbctop, sbcbot, sbctop;
            double ubot, utop, vbot, vtop, sbot, stop;
        private:
            Grid<TF>& grid;
            Fields<TF>& fields;
            std::string swboundary;
    };

    template<typename TF>
    class Thermo_dry
    {
        public:
            Thermo_dry(Grid<TF>&, Fields<TF>&, Input&);
            bool enabled() const { return swthermo; }
            void exec(double dt, cudaStream_t);      // src/thermo_dry.cxx:610-644
        private:
            Grid<TF>& grid;
            Fields<TF>& fields;
            bool swthermo;
    };

    template<typename TF>
    class Force
    {
        public:
            Force(Grid<TF>&, Fields<TF>&, Input&);
            void exec(double dt, cudaStream_t);      // src/force.cxx:610-640
            bool dpdx_on;
            double dpdx;
        private:
            Grid<TF>& grid;
            Fields<TF>& fields;
    };

    // ---- Buffer, include/buffer.h:35-70 ----------------------------------
    // Damping layer above zstart with the case's initial profiles as targets
    // (swupdate = false); the profiles are set through set_profile before
    // the first step.
    template<typename TF>
    class Buffer
    {
        public:
            Buffer(Grid<TF>&, Fields<TF>&, Input&);
            void create();                           // src/buffer.cxx:100-130
            void set_profile(const std::string& name, const double* prof);
            void exec(cudaStream_t);                 // src/buffer.cxx:160-200
            bool swbuffer;
            double zstart, sigma, beta;
        private:
            Grid<TF>& grid;
            Fields<TF>& fields;
    };

    // ---- Advec, include/advec.h:45-70 ------------------------------------
    template<typename TF>
    class Advec
    {
        public:
            Advec(Grid<TF>&, Fields<TF>&, Input&);
            virtual ~Advec() {}
            static std::unique_ptr<Advec> factory(Grid<TF>&, Fields<TF>&, Input&);
            virtual void create(Stats<TF>&) {}
            virtual void exec(Stats<TF>&) = 0;
            virtual unsigned long get_time_limit(unsigned long idt, double dt);
            virtual double get_cfl(double dt);
            virtual int get_switch() const = 0;
            void set_stream(cudaStream_t s) { stream = s; }
        protected:
            Grid<TF>& grid;
            Fields<TF>& fields;
            double cflmax;
            const double cflmin = 1.e-5;
            cudaStream_t stream = 0;
    };

    template<typename TF>
    class Advec_2i5 : public Advec<TF>
    {
        public:
            // Reads [advec] fluxlimit_list (src/advec_2i5.cxx:36-46); th in the
            // list switches its advection to the flux limiter.
            Advec_2i5(Grid<TF>&, Fields<TF>&, Input&);
            void exec(Stats<TF>&) override;
            int get_switch() const override { return MHH_ADVEC_2I5; }
            // Vertical ghost cells Advec_2i5 asks for with this input.
            static int kgc(Input&);
    };

    template<typename TF>
    class Advec_2 : public Advec<TF>
    {
        public:
            using Advec<TF>::Advec;
            void exec(Stats<TF>&) override;
            int get_switch() const override { return MHH_ADVEC_2; }
    };

    // ---- Diff, include/diff.h:37-71 --------------------------------------
    template<typename TF>
    class Diff
    {
        public:
            Diff(Grid<TF>&, Fields<TF>&, Boundary<TF>&, Input&);
            virtual ~Diff() {}
            static std::unique_ptr<Diff> factory(Grid<TF>&, Fields<TF>&, Boundary<TF>&, Input&);
            virtual void create(Stats<TF>&, const bool) {}
            virtual void exec_viscosity(Stats<TF>&, Thermo_dry<TF>&) {}
            virtual void exec(Stats<TF>&) = 0;
            virtual unsigned long get_time_limit(unsigned long idt, double dt) = 0;
            virtual double get_dn(double dt) = 0;
            virtual int get_switch() const = 0;
            void set_stream(cudaStream_t s) { stream = s; }
            TF tPr;
        protected:
            Grid<TF>& grid;
            Fields<TF>& fields;
            Boundary<TF>& boundary;
            double dnmax;
            cudaStream_t stream = 0;
    };

    template<typename TF>
    class Diff_smag2 : public Diff<TF>
    {
        public:
            Diff_smag2(Grid<TF>&, Fields<TF>&, Boundary<TF>&, Input&);
            void exec_viscosity(Stats<TF>&, Thermo_dry<TF>&) override;
            void exec(Stats<TF>&) override;
            unsigned long get_time_limit(unsigned long idt, double dt) override;
            double get_dn(double dt) override;
            int get_switch() const override { return MHH_DIFF_SMAG2; }
    };

    template<typename TF>
    class Diff_2 : public Diff<TF>
    {
        public:
            using Diff<TF>::Diff;
            void exec(Stats<TF>&) override;
            unsigned long get_time_limit(unsigned long idt, double dt) override;
            double get_dn(double dt) override;
            int get_switch() const override { return MHH_DIFF_2; }
    };

    // ---- Pres, include/pres.h:39-85 --------------------------------------
    template<typename TF>
    class Pres
    {
        public:
            Pres(Grid<TF>&, Fields<TF>&, Input&);
            virtual ~Pres() {}
            static std::unique_ptr<Pres> factory(Grid<TF>&, Fields<TF>&, Input&);
            virtual void exec(double dt, Stats<TF>&) = 0;
            virtual TF check_divergence() = 0;
            void set_stream(cudaStream_t s) { stream = s; }
        protected:
            Grid<TF>& grid;
            Fields<TF>& fields;
            cudaStream_t stream = 0;
    };

    template<typename TF>
    class Pres_2 : public Pres<TF>
    {
        public:
            using Pres<TF>::Pres;
            void exec(double dt, Stats<TF>&) override;
            TF check_divergence() override;
    };

    // ---- Timeloop, include/timeloop.h:49-139 (RK3) -----------------------
    template<typename TF>
    class Timeloop
    {
        public:
            Timeloop(Grid<TF>&, Fields<TF>&, Input&);
            void exec(cudaStream_t);
            double get_sub_time_step() const;
            void set_time_step_limit() { idtlim = idtmax; }
            void set_time_step_limit(unsigned long lim) { idtlim = std::min(idtlim, lim); }
            void set_time_step();
            bool in_substep() const { return substep > 0; }
            // src/timeloop.cxx:179-188: status every outputiter iterations at
            // the start of a step (every substep with outputiter = 0).
            bool do_check() const { return outputiter == 0 || (iteration % outputiter == 0 && !in_substep()); }
            void step_time();
            double get_dt() const { return dt; }
            unsigned long get_idt() const { return idt; }
            unsigned long get_itime() const { return itime; }
            int get_substep() const { return substep; }
            int get_iteration() const { return iteration; }
            double get_time() const { return time; }
            void advance_substep() { substep = (substep + 1) % 3; }
            // Restart state, src/timeloop.cxx:446-529: the integer time and
            // step and the iteration; iotime = itime / 10^iotimeprec s.
            void set_state(unsigned long itime_in, unsigned long idt_in, int iteration_in);
            int get_iotime() const { return int(itime/iiotimeprec); }
        private:
            Grid<TF>& grid;
            Fields<TF>& fields;
            bool adaptivestep;
            double dt, dtmax, time;
            unsigned long itime, idt, idtmax, idtlim, iiotimeprec;
            int substep, iteration, outputiter;
    };

    // ---- Model, src/model.cxx:327-581 -------------------------------------
    template<typename TF>
    class Model
    {
        public:
            explicit Model(const std::string& ini_text);
            ~Model();
            // Grid::create with the ktot full levels, then the modules in the
            // order of src/model.cxx:109-300 (cold start).
            void init(const std::vector<double>& z);
            void set_field(const std::string& name, const double* data);
            void get_field(const std::string& name, double* data);
            // n full RK3 steps; fused = one fused tendency kernel + fused
            // pressure-gradient/RK3 per substep, else the module-by-module
            // sequence of the reference loop.
            void run_steps(int n, bool fused);
            void run_substeps(int n, bool fused);
            // Relaxation target of the buffer layer for u, v or th (kcells).
            void set_buffer_profile(const std::string& name, const double* prof);
            double get_cfl();
            double get_dn();
            double get_div();
            // Restart files in the reference's formats (src/fields.cxx:1244-1344,
            // src/field3d_io.cxx:672-752, src/timeloop.cxx:446-529,
            // src/boundary_surface.cxx:584-700) in directory dir, named by
            // iotime; save returns the iotime it wrote.
            int save(const std::string& dir);
            void load(const std::string& dir, int iotime);
            Grid<TF>& get_grid() { return *grid; }
            Fields<TF>& get_fields() { return *fields; }
            Timeloop<TF>& get_timeloop() { return *timeloop; }
            // One fused substep on `stream` (what run_substeps(1, true)
            // does); with a fixed time step it launches only stream work, so
            // it can be captured into a CUDA graph.
            void substep_fused();
            // Advances the host-side time loop by one substep without
            // launching (after the replay of a captured substep).
            void advance_substep_host();
            // The arguments of this model's fused substep (mhh_substep_begin/end)
            // and its time step, for a batched substep over many models.
            void substep_args(mhh_substep_config& c, mhh_fields& f, mhh_bcfields& b, double& dt) const;
            bool adaptive() const { return adaptive_; }
            const std::string& ini() const { return ini_text; }
            const std::vector<double>& levels() const { return z_full; }
            cudaStream_t stream = 0;
            // The status check of src/model.cxx:842-872 (when the time loop's
            // do_check is due): the CFL number of the current fields; NaN, inf
            // or a value outside [0, 10) throws Nonfinite_error ("Simulation
            // has non-finite numbers").  Synchronises the stream.
            void check_status();
        private:
            void set_time_step();
            void substep_modules();
            std::string ini_text;
            std::vector<double> z_full;
            bool adaptive_ = true;
            std::unique_ptr<Input> input;
            std::unique_ptr<Grid<TF>> grid;
            std::unique_ptr<Fields<TF>> fields;
            std::unique_ptr<Boundary<TF>> boundary;
            std::unique_ptr<Thermo_dry<TF>> thermo;
            std::unique_ptr<Force<TF>> force;
            std::unique_ptr<Buffer<TF>> buffer;
            std::unique_ptr<Advec<TF>> advec;
            std::unique_ptr<Diff<TF>> diff;
            std::unique_ptr<Pres<TF>> pres;
            std::unique_ptr<Timeloop<TF>> timeloop;
            Stats<TF> stats;
            mhh_substep_config cfg;
    };

    // A model of either precision behind one handle (the mhh_model of the C
    // entry points).
    struct ModelHandle
    {
        int prec;
        std::unique_ptr<Model<double>> m64;
        std::unique_ptr<Model<float>> m32;
        template<typename F> void visit(F&& f) { if (prec == MHH_FP64) f(*m64); else f(*m32); }
    };

    // Device bytes a model of this .ini text and ktot will allocate (fields,
    // boundary arrays and the context), from the grid alone.
    size_t estimate_model_bytes(const std::string& ini_text, int ktot, int precision);
}
