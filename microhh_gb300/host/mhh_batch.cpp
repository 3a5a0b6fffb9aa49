// mhh_batch.cpp -- batched ensembles and the serving loop on top of the
// host-layer models (no counterpart in the reference, which runs one
// simulation per process).
//
// Ensemble: members of uneven grid sizes advance together.  In graph mode
// each RK3 substep of all members is captured once into a CUDA graph (every
// member on its own stream, forked from and joined into one capture stream),
// so a substep of the whole ensemble is one graph launch; an autotuner picks
// the kernel variants and level chunks per grid size by timing.
//
// Server: simulation jobs arrive over time; a job is admitted when a slot is
// free and its estimated device memory fits the budget, gets its own stream
// and a captured RK3 step, and its steps interleave with those of the other
// active jobs, so the device overlaps them.  FIFO mode runs the same jobs one
// after another for comparison.  Every job runs the same kernels with the same
// arguments in both modes, so its result does not depend on the mix.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <thread>
#include <tuple>
#include <type_traits>
#include <vector>

#include <cuda_runtime.h>

#include "mhh_host.h"
#include "mhh_batch.h"

namespace mhh_host
{
    namespace
    {
        void cuda_ok(cudaError_t e, const char* what)
        {
            if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
        }

        // One RK3 step of one model captured as three graphs (one per substep).
        struct StepGraphs
        {
            cudaGraphExec_t exec[3] = {nullptr, nullptr, nullptr};
            long long kernels = 0;    // kernel launches in one replayed step
            bool ready = false;
            void destroy()
            {
                for (auto& e : exec) if (e) { cudaGraphExecDestroy(e); e = nullptr; }
                ready = false;
            }
        };

        // Captures the next full RK3 step of h on stream s.  The capture
        // advances the host-side time loop (the substeps are issued into the
        // graphs), so the caller launches the graphs once without advancing.
        void capture_step(ModelHandle& h, cudaStream_t s, StepGraphs& g)
        {
            g.destroy();
            const long long n0 = mhh_launch_count();
            for (int q=0; q<3; ++q)
            {
                cudaGraph_t graph = nullptr;
                cuda_ok(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "begin capture");
                try
                {
                    h.visit([&](auto& m) { m.stream = s; m.substep_fused(); });
                }
                catch (...)
                {
                    cudaStreamEndCapture(s, &graph);
                    if (graph) cudaGraphDestroy(graph);
                    throw;
                }
                cuda_ok(cudaStreamEndCapture(s, &graph), "end capture");
                const cudaError_t e = cudaGraphInstantiate(&g.exec[q], graph, 0);
                cudaGraphDestroy(graph);
                cuda_ok(e, "graph instantiate");
            }
            g.kernels = mhh_launch_count() - n0;
            mhh_launch_count_add(-g.kernels);    // captured, not yet run
            g.ready = true;
        }

        void launch_step(StepGraphs& g, cudaStream_t s)
        {
            for (int q=0; q<3; ++q) cuda_ok(cudaGraphLaunch(g.exec[q], s), "graph launch");
            mhh_launch_count_add(g.kernels);
        }

        void advance_step_host(ModelHandle& h)
        {
            h.visit([](auto& m) { for (int q=0; q<3; ++q) m.advance_substep_host(); });
        }

        bool has_fixed_step(ModelHandle& h)
        {
            bool fixed = false;
            h.visit([&](auto& m) { fixed = !m.adaptive(); });
            return fixed;
        }

        mhh_ctx* ctx_of(ModelHandle& h)
        {
            mhh_ctx* c = nullptr;
            h.visit([&](auto& m) { c = m.get_grid().ctx(); });
            return c;
        }

        double now_s()
        {
            using namespace std::chrono;
            return duration<double>(steady_clock::now().time_since_epoch()).count();
        }
    }

    // ---------------------------------------------------------------------
    // Ensemble
    // ---------------------------------------------------------------------
    class Ensemble
    {
        public:
            Ensemble()
            {
                cuda_ok(cudaStreamCreateWithFlags(&main, cudaStreamNonBlocking), "stream");
                cuda_ok(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "event");
            }
            ~Ensemble()
            {
                cudaStreamSynchronize(main);
                for (auto s : streams) cudaStreamSynchronize(s);
                drop_graphs();
                // The members outlive the ensemble: back to the default stream.
                for (auto* h : members) h->visit([](auto& m) { m.stream = 0; });
                for (auto s : streams) cudaStreamDestroy(s);
                for (auto e : joins) cudaEventDestroy(e);
                cudaEventDestroy(fork);
                cudaStreamDestroy(main);
            }

            void add(ModelHandle* h)
            {
                cudaStream_t s;
                cudaEvent_t e;
                cuda_ok(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream");
                cuda_ok(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
                members.push_back(h);
                streams.push_back(s);
                joins.push_back(e);
                drop_graphs();
            }

            void run_steps(int n, int mode)
            {
                if (mode == MHH_ENS_SEQUENTIAL)
                {
                    for (auto* h : members)
                        h->visit([&](auto& m) { m.stream = main; m.run_steps(n, true); });
                    return;
                }
                if (mode == MHH_ENS_STREAMS)
                {
                    for (int step=0; step<n; ++step) eager_step();
                    return;
                }
                if (mode != MHH_ENS_GRAPHS && mode != MHH_ENS_BATCHED) throw std::runtime_error("unknown ensemble mode");
                for (auto* h : members)
                    if (!has_fixed_step(*h)) throw std::runtime_error("graph mode needs adaptivestep=false in every member");
                if ((mode == MHH_ENS_BATCHED) != batched) drop_graphs();
                batched = mode == MHH_ENS_BATCHED;
                int done = 0;
                if (!captured && done < n)
                {
                    // One eager step sets every kernel's attributes outside a
                    // capture; the following step is captured and launched.
                    eager_step();
                    ++done;
                    if (done < n)
                    {
                        if (batched)
                        {
                            // The plan records the members' next substeps
                            // without advancing their time loops.
                            capture_batched();
                            launch_graphs();
                            for (auto* h : members) advance_step_host(*h);
                        }
                        else
                        {
                            capture();
                            launch_graphs();
                        }
                        ++done;
                    }
                }
                for (; done < n; ++done)
                {
                    launch_graphs();
                    for (auto* h : members) advance_step_host(*h);
                }
            }

            void synchronize()
            {
                cuda_ok(cudaStreamSynchronize(main), "sync");
                for (auto s : streams) cuda_ok(cudaStreamSynchronize(s), "sync");
            }

            std::string autotune();

        private:
            void eager_step()
            {
                // Fork from the main stream so that earlier sequential work
                // (on main) is ordered before the members' streams.
                cuda_ok(cudaEventRecord(fork, main), "record");
                for (size_t i=0; i<members.size(); ++i) cuda_ok(cudaStreamWaitEvent(streams[i], fork, 0), "wait");
                for (int q=0; q<3; ++q)
                    for (size_t i=0; i<members.size(); ++i)
                        members[i]->visit([&](auto& m) { m.stream = streams[i]; m.substep_fused(); });
                for (size_t i=0; i<members.size(); ++i)
                {
                    cuda_ok(cudaEventRecord(joins[i], streams[i]), "record");
                    cuda_ok(cudaStreamWaitEvent(main, joins[i], 0), "wait");
                }
            }

            // Batch plans over the members (mhh_batch_create), one per grid
            // size: within a plan every stage is one kernel over all its
            // members, and the plans run as parallel branches of the graph,
            // so that members of one size do not wait at every stage for the
            // tails of the other sizes.  A substep of the whole ensemble is
            // one graph whose kernel nodes are the batched stages.
            void capture_batched()
            {
                drop_graphs();
                std::map<std::tuple<int, int, int>, std::vector<size_t>> buckets;
                for (size_t i=0; i<members.size(); ++i)
                {
                    mhh_grid g;
                    members[i]->visit([&](auto& m) { g = m.get_grid().get_grid_data(); });
                    buckets[std::make_tuple(g.itot, g.jtot, g.ktot)].push_back(i);
                }
                cuda_ok(cudaStreamSynchronize(main), "sync");
                for (auto st : streams) cuda_ok(cudaStreamSynchronize(st), "sync");
                for (auto& kv : buckets)
                {
                    const size_t n = kv.second.size();
                    std::vector<mhh_ctx*> ctx(n);
                    std::vector<mhh_substep_config> cfg(n);
                    std::vector<mhh_fields> f(n);
                    std::vector<mhh_bcfields> bc(n);
                    std::vector<double> dt(n);
                    for (size_t q=0; q<n; ++q)
                    {
                        ModelHandle* h = members[kv.second[q]];
                        ctx[q] = ctx_of(*h);
                        h->visit([&](auto& m) { m.substep_args(cfg[q], f[q], bc[q], dt[q]); });
                    }
                    mhh_batch* p = nullptr;
                    if (mhh_batch_create((int)n, ctx.data(), cfg.data(), f.data(), bc.data(), dt.data(), &p) != MHH_OK)
                        throw std::runtime_error(std::string("batch plan: ") + mhh_last_error());
                    plans.push_back(p);
                }
                gkernels = 0;
                for (int q=0; q<3; ++q)
                {
                    for (auto* p : plans)
                    {
                        int nl = 0;
                        mhh_batch_launches(p, q, &nl);
                        gkernels += nl;
                    }
                    cudaGraph_t graph = nullptr;
                    cuda_ok(cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal), "begin capture");
                    int rc = MHH_OK;
                    cuda_ok(cudaEventRecord(fork, main), "record");
                    for (size_t b=0; b<plans.size() && rc == MHH_OK; ++b)
                    {
                        cuda_ok(cudaStreamWaitEvent(streams[b], fork, 0), "wait");
                        rc = mhh_batch_substep(plans[b], q, streams[b]);
                        cuda_ok(cudaEventRecord(joins[b], streams[b]), "record");
                        cuda_ok(cudaStreamWaitEvent(main, joins[b], 0), "wait");
                    }
                    cuda_ok(cudaStreamEndCapture(main, &graph), "end capture");
                    if (rc != MHH_OK)
                    {
                        if (graph) cudaGraphDestroy(graph);
                        throw std::runtime_error(std::string("batch substep: ") + mhh_last_error());
                    }
                    const cudaError_t e = cudaGraphInstantiate(&gexec[q], graph, 0);
                    cudaGraphDestroy(graph);
                    cuda_ok(e, "graph instantiate");
                }
                mhh_launch_count_add(-gkernels);   // captured, not yet run
                captured = true;
            }

            void capture()
            {
                drop_graphs();
                const long long n0 = mhh_launch_count();
                for (int q=0; q<3; ++q)
                {
                    cudaGraph_t graph = nullptr;
                    cuda_ok(cudaStreamBeginCapture(main, cudaStreamCaptureModeThreadLocal), "begin capture");
                    try
                    {
                        cuda_ok(cudaEventRecord(fork, main), "record");
                        for (size_t i=0; i<members.size(); ++i)
                        {
                            cuda_ok(cudaStreamWaitEvent(streams[i], fork, 0), "wait");
                            members[i]->visit([&](auto& m) { m.stream = streams[i]; m.substep_fused(); });
                            cuda_ok(cudaEventRecord(joins[i], streams[i]), "record");
                            cuda_ok(cudaStreamWaitEvent(main, joins[i], 0), "wait");
                        }
                    }
                    catch (...)
                    {
                        cudaStreamEndCapture(main, &graph);
                        if (graph) cudaGraphDestroy(graph);
                        throw;
                    }
                    cuda_ok(cudaStreamEndCapture(main, &graph), "end capture");
                    const cudaError_t e = cudaGraphInstantiate(&gexec[q], graph, 0);
                    cudaGraphDestroy(graph);
                    cuda_ok(e, "graph instantiate");
                }
                gkernels = mhh_launch_count() - n0;
                mhh_launch_count_add(-gkernels);
                captured = true;
            }

            void launch_graphs()
            {
                for (int q=0; q<3; ++q) cuda_ok(cudaGraphLaunch(gexec[q], main), "graph launch");
                mhh_launch_count_add(gkernels);
            }

            void drop_graphs()
            {
                for (auto& g : gexec) if (g) { cudaGraphExecDestroy(g); g = nullptr; }
                for (auto* p : plans) mhh_batch_destroy(p);
                plans.clear();
                captured = false;
            }

            std::vector<ModelHandle*> members;
            std::vector<cudaStream_t> streams;
            std::vector<cudaEvent_t> joins;
            cudaStream_t main = nullptr;
            cudaEvent_t fork = nullptr;
            cudaGraphExec_t gexec[3] = {nullptr, nullptr, nullptr};
            long long gkernels = 0;
            bool captured = false;
            bool batched = false;
            std::vector<mhh_batch*> plans;
    };

    // Times a scratch copy of one member per grid size under each candidate
    // kernel choice and applies the fastest to the members of that size.
    std::string Ensemble::autotune()
    {
        synchronize();
        std::map<std::tuple<int, int, int, int>, std::vector<ModelHandle*>> groups;
        for (auto* h : members)
        {
            mhh_grid g;
            h->visit([&](auto& m) { g = m.get_grid().get_grid_data(); });
            groups[std::make_tuple(g.itot, g.jtot, g.ktot, h->prec)].push_back(h);
        }
        cudaEvent_t e0, e1;
        cuda_ok(cudaEventCreate(&e0), "event");
        cuda_ok(cudaEventCreate(&e1), "event");
        std::ostringstream rep;
        for (auto& kv : groups)
        {
            ModelHandle* ref = kv.second.front();
            ModelHandle scratch;
            scratch.prec = ref->prec;
            ref->visit([&](auto& m)
            {
                using M = std::decay_t<decltype(m)>;
                auto sm = std::make_unique<M>(m.ini());
                sm->init(m.levels());
                // Start from the member's state so that every branch is the one
                // the member takes (the member itself is not advanced).
                const mhh_fields src = m.get_fields().dev(), dst = sm->get_fields().dev();
                const mhh_grid gd = m.get_grid().get_grid_data();
                const size_t bytes = size_t(gd.ncells)*(ref->prec == MHH_FP64 ? 8 : 4);
                const void* s4[4] = {src.u, src.v, src.w, src.s};
                void* d4[4] = {dst.u, dst.v, dst.w, dst.s};
                for (int q=0; q<4; ++q) if (s4[q] && d4[q]) cuda_ok(cudaMemcpy(d4[q], s4[q], bytes, cudaMemcpyDeviceToDevice), "copy");
                if constexpr (std::is_same_v<M, Model<double>>) scratch.m64 = std::move(sm);
                else scratch.m32 = std::move(sm);
            });
            mhh_ctx* c = ctx_of(scratch);
            auto time_step = [&]() -> double
            {
                scratch.visit([&](auto& m) { m.stream = main; m.run_steps(1, true); });
                cuda_ok(cudaEventRecord(e0, main), "record");
                scratch.visit([&](auto& m) { m.run_steps(2, true); });
                cuda_ok(cudaEventRecord(e1, main), "record");
                cuda_ok(cudaEventSynchronize(e1), "sync");
                float ms = 0.f;
                cuda_ok(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
                return ms/2.;
            };
            struct Cand { const char* opt; const char* chunk; int v, k; };
            const Cand tcand[] = {{"tendency_kernel", "tendency_kchunk", 0, 0}, {"tendency_kernel", "tendency_kchunk", 2, 8},
                                  {"tendency_kernel", "tendency_kchunk", 2, 16}, {"tendency_kernel", "tendency_kchunk", 2, 32},
                                  {"tendency_kernel", "tendency_kchunk", 2, 64}};
            const Cand vcand[] = {{"viscosity_kernel", "viscosity_kchunk", 0, 0}, {"viscosity_kernel", "viscosity_kchunk", 1, 8},
                                  {"viscosity_kernel", "viscosity_kchunk", 1, 16}, {"viscosity_kernel", "viscosity_kchunk", 1, 32},
                                  {"viscosity_kernel", "viscosity_kchunk", 1, 64}};
            auto pick = [&](const Cand* cands, int n, int& bv, int& bk, double& bt)
            {
                bt = 1e30;
                for (int q=0; q<n; ++q)
                {
                    check(mhh_ctx_set_option(c, cands[q].opt, cands[q].v), "set option");
                    check(mhh_ctx_set_option(c, cands[q].chunk, cands[q].k), "set option");
                    const double t = time_step();
                    if (t < bt) { bt = t; bv = cands[q].v; bk = cands[q].k; }
                }
                check(mhh_ctx_set_option(c, cands[0].opt, bv), "set option");
                check(mhh_ctx_set_option(c, cands[0].chunk, bk), "set option");
            };
            int tv = 0, tk = 0, vv = 0, vk = 0;
            double tt = 0., vt = 0.;
            pick(tcand, 5, tv, tk, tt);
            pick(vcand, 5, vv, vk, vt);
            for (auto* h : kv.second)
            {
                mhh_ctx* mc = ctx_of(*h);
                check(mhh_ctx_set_option(mc, "tendency_kernel", tv), "set option");
                check(mhh_ctx_set_option(mc, "tendency_kchunk", tk), "set option");
                check(mhh_ctx_set_option(mc, "viscosity_kernel", vv), "set option");
                check(mhh_ctx_set_option(mc, "viscosity_kchunk", vk), "set option");
            }
            rep << std::get<0>(kv.first) << "x" << std::get<1>(kv.first) << "x" << std::get<2>(kv.first)
                << ": tendency " << tv << "/" << tk << " viscosity " << vv << "/" << vk
                << " (" << vt << " ms/step); ";
            cuda_ok(cudaStreamSynchronize(main), "sync");
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        drop_graphs();
        return rep.str();
    }

    // ---------------------------------------------------------------------
    // Server
    // ---------------------------------------------------------------------
    class Server
    {
        public:
            Server(double budget, int max_active) : budget(budget), max_active(max_active) {}
            ~Server() { for (auto& j : jobs) retire_now(j, false); }

            int submit(const char* ini, const double* z, int ktot, int prec, int nsteps, double arrival, int keep)
            {
                if (prec != MHH_FP64 && prec != MHH_FP32) throw std::runtime_error("precision must be 64 or 32");
                if (nsteps < 1) throw std::runtime_error("a job needs at least one step");
                Job j;
                j.ini = ini;
                j.z.assign(z, z + ktot);
                j.prec = prec;
                j.nsteps = nsteps;
                j.arrival = arrival;
                j.keep = keep != 0;
                j.est = (double)estimate_model_bytes(j.ini, ktot, prec);
                {
                    Input in(j.ini);
                    j.cells = double(in.get_item<int>("grid", "itot", ""))*in.get_item<int>("grid", "jtot", "")*ktot;
                }
                jobs.push_back(std::move(j));
                return (int)jobs.size() - 1;
            }

            void set_initial(int id, const char* name, const double* data)
            {
                Job& j = job(id);
                // Size from the grid of the .ini text.
                Input in(j.ini);
                const std::string swadvec = in.get_item<std::string>("advec", "swadvec", "", "2");
                const int gc = swadvec == "2i5" ? 3 : 1;
                const int kgc = swadvec == "2i5" && !in.get_list("advec", "fluxlimit_list", "", {}).empty() ? 2 : 1;
                const size_t n = size_t(in.get_item<int>("grid", "itot", "") + 2*gc)
                               * size_t(in.get_item<int>("grid", "jtot", "") + 2*gc) * (j.z.size() + 2*kgc);
                j.init[name] = std::vector<double>(data, data + n);
            }

            void run(int mode)
            {
                if (mode != MHH_SERVE_FIFO && mode != MHH_SERVE_CONTINUOUS) throw std::runtime_error("unknown server mode");
                for (auto& j : jobs) { retire_now(j, false); j.t_admit = j.t_finish = -1.; j.out.clear(); j.issued = 0; }
                progress.clear();
                std::vector<int> order(jobs.size());
                for (size_t q=0; q<order.size(); ++q) order[q] = (int)q;
                std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return jobs[a].arrival < jobs[b].arrival; });
                used = 0.; peak = 0.;
                t0 = now_s();
                if (mode == MHH_SERVE_FIFO)
                {
                    for (int id : order)
                    {
                        Job& j = jobs[id];
                        wait_until(j.arrival);
                        admit(j);
                        while (j.issued < j.nsteps) issue_step(j);
                        // Completion time of every step, in order.
                        while (!j.inflight.empty())
                        {
                            cuda_ok(cudaEventSynchronize(j.inflight.front()), "event sync");
                            step_done(j);
                        }
                        retire_now(j, true);
                    }
                    return;
                }
                size_t next = 0;
                std::vector<int> active;
                size_t finished = 0;
                while (finished < jobs.size())
                {
                    const double t = now_s() - t0;
                    // Admission: arrived jobs in arrival order while a slot and
                    // the memory budget allow.
                    while (next < order.size() && jobs[order[next]].arrival <= t && (int)active.size() < max_active
                           && (active.empty() || used + jobs[order[next]].est <= budget))
                    {
                        Job& j = jobs[order[next]];
                        admit(j);
                        active.push_back(order[next]);
                        ++next;
                    }
                    // Issue: a few steps in flight per job, round robin.
                    bool progressed = false;
                    for (int id : active)
                    {
                        Job& j = jobs[id];
                        while (j.issued < j.nsteps && j.inflight.size() < 3) { issue_step(j); progressed = true; }
                    }
                    // Completion.
                    for (size_t q=0; q<active.size();)
                    {
                        Job& j = jobs[active[q]];
                        while (!j.inflight.empty() && cudaEventQuery(j.inflight.front()) == cudaSuccess)
                        {
                            step_done(j);
                            progressed = true;
                        }
                        if (j.issued == j.nsteps && j.inflight.empty())
                        {
                            retire_now(j, true);
                            active.erase(active.begin() + q);
                            ++finished;
                            progressed = true;
                        }
                        else
                            ++q;
                    }
                    if (!progressed)
                    {
                        // Nothing completed: poll again shortly.  Blocking on
                        // one job's event would leave the other jobs without
                        // new work until that (possibly long) step ends.
                        if (!active.empty())
                            std::this_thread::sleep_for(std::chrono::microseconds(20));
                        else if (next < order.size())
                            wait_until(jobs[order[next]].arrival);
                    }
                }
            }

            void times(int id, double* a, double* ad, double* f)
            {
                Job& j = job(id);
                *a = j.arrival; *ad = j.t_admit; *f = j.t_finish;
            }

            void result(int id, const char* name, double* data)
            {
                Job& j = job(id);
                auto it = j.out.find(name);
                if (it == j.out.end()) throw std::runtime_error("no kept result of that name (submit with keep = 1)");
                std::copy(it->second.begin(), it->second.end(), data);
            }

            double peak_bytes() const { return peak; }
            const std::vector<std::pair<double, double>>& progress_log() const { return progress; }

        private:
            struct Job
            {
                std::string ini;
                std::vector<double> z;
                int prec = MHH_FP32, nsteps = 1;
                double arrival = 0., est = 0., cells = 0.;
                bool keep = false;
                std::map<std::string, std::vector<double>> init;
                std::unique_ptr<ModelHandle> h;
                cudaStream_t stream = nullptr;
                StepGraphs graphs;
                int issued = 0;
                std::deque<cudaEvent_t> inflight;
                double t_admit = -1., t_finish = -1.;
                std::map<std::string, std::vector<double>> out;
            };

            // A step of j completed (its event has been seen): log the time
            // and the cells it advanced.
            void step_done(Job& j)
            {
                release_event(j.inflight.front());
                j.inflight.pop_front();
                progress.emplace_back(now_s() - t0, j.cells);
            }

            Job& job(int id)
            {
                if (id < 0 || id >= (int)jobs.size()) throw std::runtime_error("no such job");
                return jobs[id];
            }

            void wait_until(double t)
            {
                for (;;)
                {
                    const double d = t - (now_s() - t0);
                    if (d <= 0.) return;
                    std::this_thread::sleep_for(std::chrono::duration<double>(std::min(d, 0.01)));
                }
            }

            void admit(Job& j)
            {
                j.h = std::make_unique<ModelHandle>();
                j.h->prec = j.prec;
                if (j.prec == MHH_FP64) { j.h->m64 = std::make_unique<Model<double>>(j.ini); j.h->m64->init(j.z); }
                else { j.h->m32 = std::make_unique<Model<float>>(j.ini); j.h->m32->init(j.z); }
                for (auto& kv : j.init) j.h->visit([&](auto& m) { m.set_field(kv.first, kv.second.data()); });
                if (!has_fixed_step(*j.h)) throw std::runtime_error("served jobs need adaptivestep=false");
                cuda_ok(cudaStreamCreateWithFlags(&j.stream, cudaStreamNonBlocking), "stream");
                j.h->visit([&](auto& m) { m.stream = j.stream; });
                j.t_admit = now_s() - t0;
                used += j.est;
                peak = std::max(peak, used);
            }

            // One RK3 step: the first eagerly, the second captured (and run),
            // the rest replayed.
            void issue_step(Job& j)
            {
                if (j.issued == 0)
                    j.h->visit([&](auto& m) { m.run_steps(1, true); });
                else if (!j.graphs.ready)
                {
                    capture_step(*j.h, j.stream, j.graphs);
                    launch_step(j.graphs, j.stream);
                }
                else
                {
                    launch_step(j.graphs, j.stream);
                    advance_step_host(*j.h);
                }
                cudaEvent_t e = take_event();
                cuda_ok(cudaEventRecord(e, j.stream), "record");
                j.inflight.push_back(e);
                ++j.issued;
            }

            void retire_now(Job& j, bool finished)
            {
                if (!j.h) return;
                cudaStreamSynchronize(j.stream);
                for (auto e : j.inflight) release_event(e);
                j.inflight.clear();
                if (finished && j.keep)
                    for (const char* n : {"u", "v", "w", "th"})
                    {
                        bool has = true;
                        j.h->visit([&](auto& m) { has = n[0] != 't' || m.get_fields().sp.count("th"); });
                        if (!has) continue;
                        mhh_grid gd;
                        j.h->visit([&](auto& m) { gd = m.get_grid().get_grid_data(); });
                        std::vector<double> buf(gd.ncells);
                        j.h->visit([&](auto& m) { m.get_field(n, buf.data()); });
                        j.out[n] = std::move(buf);
                    }
                j.graphs.destroy();
                j.h.reset();
                cudaStreamDestroy(j.stream);
                j.stream = nullptr;
                used -= j.est;
                if (finished) j.t_finish = now_s() - t0;
            }

            cudaEvent_t take_event()
            {
                if (!pool.empty()) { cudaEvent_t e = pool.back(); pool.pop_back(); return e; }
                cudaEvent_t e;
                cuda_ok(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
                return e;
            }
            void release_event(cudaEvent_t e) { pool.push_back(e); }

            double budget;
            int max_active;
            std::vector<Job> jobs;
            std::vector<cudaEvent_t> pool;
            std::vector<std::pair<double, double>> progress;   // (time, cells) per completed step
            double used = 0., peak = 0., t0 = 0.;
    };
}

// ---------------------------------------------------------------------------
// C entry points (include/mhh_batch.h)
// ---------------------------------------------------------------------------
namespace
{
    thread_local std::string g_batch_error;

    template<typename F>
    int guard_b(F&& f)
    {
        try { f(); return MHH_OK; }
        catch (std::exception& e) { g_batch_error = e.what(); return MHH_ERR_ARG; }
    }
}

extern "C" {

const char* mhh_batch_last_error(void) { return g_batch_error.c_str(); }

int mhh_ensemble_create(mhh_ensemble** out)
{
    if (!out) { g_batch_error = "NULL argument"; return MHH_ERR_ARG; }
    return guard_b([&] { *out = reinterpret_cast<mhh_ensemble*>(new mhh_host::Ensemble()); });
}

int mhh_ensemble_add(mhh_ensemble* e, mhh_model* m)
{
    if (!e || !m) { g_batch_error = "NULL argument"; return MHH_ERR_ARG; }
    return guard_b([&] { reinterpret_cast<mhh_host::Ensemble*>(e)->add(reinterpret_cast<mhh_host::ModelHandle*>(m)); });
}

int mhh_ensemble_autotune(mhh_ensemble* e, char* report, int report_len)
{
    if (!e) { g_batch_error = "NULL argument"; return MHH_ERR_ARG; }
    return guard_b([&]
    {
        const std::string r = reinterpret_cast<mhh_host::Ensemble*>(e)->autotune();
        if (report && report_len > 0)
        {
            std::strncpy(report, r.c_str(), report_len - 1);
            report[report_len - 1] = 0;
        }
    });
}

int mhh_ensemble_run_steps(mhh_ensemble* e, int n, int mode)
{
    if (!e) { g_batch_error = "NULL argument"; return MHH_ERR_ARG; }
    return guard_b([&] { reinterpret_cast<mhh_host::Ensemble*>(e)->run_steps(n, mode); });
}

int mhh_ensemble_synchronize(mhh_ensemble* e)
{
    if (!e) { g_batch_error = "NULL argument"; return MHH_ERR_ARG; }
    return guard_b([&] { reinterpret_cast<mhh_host::Ensemble*>(e)->synchronize(); });
}

int mhh_ensemble_destroy(mhh_ensemble* e)
{
    delete reinterpret_cast<mhh_host::Ensemble*>(e);
    return MHH_OK;
}

int mhh_server_create(double budget_bytes, int max_active, mhh_server** out)
{
    if (!out || budget_bytes <= 0. || max_active < 1) { g_batch_error = "bad argument"; return MHH_ERR_ARG; }
    return guard_b([&] { *out = reinterpret_cast<mhh_server*>(new mhh_host::Server(budget_bytes, max_active)); });
}

int mhh_server_submit(mhh_server* s, const char* ini_text, const double* z, int ktot, int precision, int nsteps,
                      double arrival_s, int keep, int* job)
{
    if (!s || !ini_text || !z || !job) { g_batch_error = "NULL argument"; return MHH_ERR_ARG; }
    return guard_b([&] { *job = reinterpret_cast<mhh_host::Server*>(s)->submit(ini_text, z, ktot, precision, nsteps,
                                                                               arrival_s, keep); });
}

int mhh_server_set_initial(mhh_server* s, int job, const char* name, const double* data)
{
    if (!s || !name || !data) { g_batch_error = "NULL argument"; return MHH_ERR_ARG; }
    return guard_b([&] { reinterpret_cast<mhh_host::Server*>(s)->set_initial(job, name, data); });
}

int mhh_server_run(mhh_server* s, int mode)
{
    if (!s) { g_batch_error = "NULL argument"; return MHH_ERR_ARG; }
    return guard_b([&] { reinterpret_cast<mhh_host::Server*>(s)->run(mode); });
}

int mhh_server_job_times(mhh_server* s, int job, double* arrival, double* admit, double* finish)
{
    if (!s || !arrival || !admit || !finish) { g_batch_error = "NULL argument"; return MHH_ERR_ARG; }
    return guard_b([&] { reinterpret_cast<mhh_host::Server*>(s)->times(job, arrival, admit, finish); });
}

int mhh_server_get_result(mhh_server* s, int job, const char* name, double* data)
{
    if (!s || !name || !data) { g_batch_error = "NULL argument"; return MHH_ERR_ARG; }
    return guard_b([&] { reinterpret_cast<mhh_host::Server*>(s)->result(job, name, data); });
}

int mhh_server_peak_bytes(mhh_server* s, double* bytes)
{
    if (!s || !bytes) { g_batch_error = "NULL argument"; return MHH_ERR_ARG; }
    *bytes = reinterpret_cast<mhh_host::Server*>(s)->peak_bytes();
    return MHH_OK;
}

int mhh_server_progress(mhh_server* s, double* times, double* cells, int max, int* count)
{
    if (!s || !count) { g_batch_error = "NULL argument"; return MHH_ERR_ARG; }
    const auto& log = reinterpret_cast<mhh_host::Server*>(s)->progress_log();
    *count = (int)log.size();
    for (int q=0; q<std::min(max, (int)log.size()); ++q)
    {
        if (times) times[q] = log[q].first;
        if (cells) cells[q] = log[q].second;
    }
    return MHH_OK;
}

int mhh_server_destroy(mhh_server* s)
{
    delete reinterpret_cast<mhh_host::Server*>(s);
    return MHH_OK;
}

}
