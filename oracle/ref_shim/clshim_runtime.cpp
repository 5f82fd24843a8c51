/*
 * clshim_runtime.cpp -- NDRange runner for the reference kernels compiled on the CPU.
 * TEST INFRASTRUCTURE (oracle/_ref only).  Work-items of a work-group run as ucontext
 * fibers; barrier() yields to the group scheduler, which resumes every live work-item
 * once per round, so all work-items reach barrier k before any passes it.
 */
#include "clshim.hpp"

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

void run_ndrange(size_t global, size_t local, bool fibers, const std::function<void()>& body) {
    if (local == 0) local = 1;
    const size_t groups = (global + local - 1) / local;
    if (!fibers) {
        for (size_t g = 0; g < groups; ++g)
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
    for (size_t g = 0; g < groups; ++g) {
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
