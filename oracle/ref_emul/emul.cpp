// emul.cpp — fiber scheduler of cuda_emul.hpp.  TEST INFRASTRUCTURE ONLY.
#include "cuda_emul.hpp"

#include <stdexcept>

namespace emu {

Fiber *g_cur = nullptr;
uint3 g_block_idx{0, 0, 0}, g_block_dim{1, 1, 1}, g_grid_dim{1, 1, 1};

namespace {
constexpr size_t kStack = 64 * 1024;
ucontext_t g_sched;
std::vector<Fiber> g_fibers;
const std::function<void()> *g_body = nullptr;

void entry()
{
    (*g_body)();
    g_cur->done = true;  // returning resumes g_sched through uc_link
}
}  // namespace

void syncthreads()
{
    g_cur->at_barrier = true;
    swapcontext(&g_cur->ctx, &g_sched);
}

void launch(unsigned grid, unsigned block, const std::function<void()> &body)
{
    if (block == 0 || block > 1024) throw std::runtime_error("emulated launch: bad block size");
    if (g_fibers.size() < block) g_fibers.resize(block);
    g_body = &body;
    g_grid_dim = uint3{grid, 1, 1};
    g_block_dim = uint3{block, 1, 1};
    for (unsigned b = 0; b < grid; ++b) {
        g_block_idx = uint3{b, 0, 0};
        for (unsigned t = 0; t < block; ++t) {
            Fiber &f = g_fibers[t];
            if (f.stack.size() < kStack) f.stack.resize(kStack);
            getcontext(&f.ctx);
            f.ctx.uc_stack.ss_sp = f.stack.data();
            f.ctx.uc_stack.ss_size = f.stack.size();
            f.ctx.uc_link = &g_sched;
            makecontext(&f.ctx, entry, 0);
            f.tid = uint3{t, 0, 0};
            f.done = false;
            f.at_barrier = false;
        }
        for (;;) {
            for (unsigned t = 0; t < block; ++t) {
                Fiber &f = g_fibers[t];
                if (f.done || f.at_barrier) continue;
                g_cur = &f;
                swapcontext(&g_sched, &f.ctx);
            }
            bool waiting = false;
            for (unsigned t = 0; t < block; ++t) {
                if (g_fibers[t].at_barrier) {
                    g_fibers[t].at_barrier = false;
                    waiting = true;
                }
            }
            if (!waiting) break;
        }
    }
    g_cur = nullptr;
}

}  // namespace emu
