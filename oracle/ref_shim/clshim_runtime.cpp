/*
 * clshim_runtime.cpp -- NDRange runner for the reference kernels compiled on the CPU.
 * TEST INFRASTRUCTURE (oracle/_ref only).  Work-items of a work-group run as ucontext
 * fibers; barrier() yields to the group scheduler, which resumes every live work-item
 * once per round, so all work-items reach barrier k before any passes it.  Work-groups run
 * on the host's threads.
 */
#include "clshim.hpp"

#include <algorithm>
#include <cstdlib>
#include <thread>

namespace clshim {
int g_particle_count = 0;
int g_boundary_particle_count = 0;
float g_support_radius = 0.f;
float g_particle_mass = 0.f;
float g_rest_density = 0.f;
float g_cell_size = 0.f;
float g_grid_size = 0.f;
int g_cells_per_side = 0;

thread_local WorkItem* tl_cur = nullptr;

namespace {
struct Fiber {
    ucontext_t ctx;
    WorkItem wi;
    bool done;
};
thread_local ucontext_t* tl_sched = nullptr;
thread_local Fiber* tl_fiber = nullptr;
thread_local const std::function<void()>* tl_body = nullptr;

void trampoline() {
    Fiber* f = tl_fiber;
    (*tl_body)();
    f->done = true;
}
}  // namespace

void barrier_impl() {
    if (!tl_fiber) {
        std::fprintf(stderr, "clshim: barrier() in a kernel launched without fibers\n");
        std::abort();
    }
    swapcontext(&tl_fiber->ctx, tl_sched);
}

namespace {
/* work-groups [g0, g1) on the calling thread */
void run_groups(size_t g0, size_t g1, size_t local, bool fibers, const std::function<void()>& body) {
    if (!fibers) {
        for (size_t g = g0; g < g1; ++g)
            for (size_t l = 0; l < local; ++l) {
                WorkItem wi{g * local + l, l, local, g};
                tl_cur = &wi;
                body();
            }
        tl_cur = nullptr;
        return;
    }
    const size_t kStack = 128 * 1024;
    std::vector<Fiber> fs(local);
    std::vector<std::vector<char>> stacks(local, std::vector<char>(kStack));
    ucontext_t sched;
    tl_sched = &sched;
    tl_body = &body;
    for (size_t g = g0; g < g1; ++g) {
        for (size_t l = 0; l < local; ++l) {
            fs[l].wi = WorkItem{g * local + l, l, local, g};
            fs[l].done = false;
            getcontext(&fs[l].ctx);
            fs[l].ctx.uc_stack.ss_sp = stacks[l].data();
            fs[l].ctx.uc_stack.ss_size = kStack;
            fs[l].ctx.uc_link = &sched;
            makecontext(&fs[l].ctx, trampoline, 0);
        }
        for (;;) {
            bool live = false;
            for (size_t l = 0; l < local; ++l) {
                if (fs[l].done) continue;
                tl_cur = &fs[l].wi;
                tl_fiber = &fs[l];
                swapcontext(&sched, &fs[l].ctx);
                if (!fs[l].done) live = true;
            }
            if (!live) break;
        }
    }
    tl_fiber = nullptr;
    tl_cur = nullptr;
    tl_body = nullptr;
    tl_sched = nullptr;
}

int host_threads() {
    const char* e = std::getenv("SPH_REF_THREADS");
    const int t = e ? std::atoi(e) : (int)std::thread::hardware_concurrency();
    return t < 1 ? 1 : t;
}
}  // namespace

void* group_local(int slot, size_t bytes) {
    thread_local std::vector<unsigned char> bufs[8];
    std::vector<unsigned char>& b = bufs[slot & 7];
    if (b.size() < bytes) b.resize(bytes);
    return b.data();
}

/* Work-groups are independent (the kernels use no global atomics), so they are spread over
 * the host's threads (SPH_REF_THREADS, default all); the work-items of a group stay on one
 * thread, as fibers when the kernel has barriers, sharing that thread's group_local memory. */
void run_ndrange(size_t global, size_t local, bool fibers, const std::function<void()>& body) {
    if (local == 0) local = 1;
    const size_t groups = (global + local - 1) / local;
    const size_t t = std::min<size_t>((size_t)host_threads(), groups / 16 + 1);
    if (t <= 1) {
        run_groups(0, groups, local, fibers, body);
        return;
    }
    std::vector<std::thread> th;
    const size_t chunk = (groups + t - 1) / t;
    for (size_t k = 0; k < t; ++k) {
        const size_t g0 = k * chunk, g1 = std::min(groups, g0 + chunk);
        if (g0 < g1) th.emplace_back(run_groups, g0, g1, local, fibers, std::cref(body));
    }
    for (auto& x : th) x.join();
}

void run_ndrange_2d(size_t gx, size_t gy, const std::function<void()>& body) {
    for (size_t y = 0; y < gy; ++y)
        for (size_t x = 0; x < gx; ++x) {
            WorkItem wi{x, x, gx, 0, y};
            tl_cur = &wi;
            body();
        }
    tl_cur = nullptr;
}

}  // namespace clshim
