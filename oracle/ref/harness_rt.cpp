/*
 * TEST INFRASTRUCTURE ONLY.  Runtime for the reference compiled on the CPU
 * (see shim.h): launch emulation, barrier fibers, printf guard, the
 * stream behind the fake curand_uniform_double, and the process entry
 * point that calls the reference's own main() (renamed sevc_ref_main).
 *
 * Environment:
 *   SEVC_REF_MIN_GRAINS   value for src/main.cu:49 (default 5000)
 *   SEVC_REF_RNG_SEED     seed of the synthetic stream (default 0)
 *   SEVC_REF_RNG_TABLE    file of recorded draws (raw float64, stream-major)
 *   SEVC_REF_RNG_NDRAWS   draws per stream in that file
 *   SEVC_REF_QUIET        silence printf
 */
#include <setjmp.h>
#include <ucontext.h>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <vector>

#include "../synth_rng.h"

struct sevc_dim3 { unsigned int x, y, z; };
sevc_dim3 blockIdx, threadIdx, blockDim, gridDim;

int sevc_ref_main(int argc, char const *argv[]);

/* ---------------- kernel launch emulation ---------------- */
namespace {
/* Fibers start once through makecontext/swapcontext; afterwards every
 * switch uses _setjmp/_longjmp, which do not touch the signal mask (no
 * system call per barrier). */
struct Fiber { ucontext_t ctx; jmp_buf jb; std::vector<char> stack; bool done, started; };
jmp_buf g_sched_jb;
ucontext_t g_boot;
Fiber *g_cur = nullptr;
bool g_fiber_mode = false;
const std::function<void()> *g_body = nullptr;
std::vector<Fiber> g_pool;

void fiber_entry()
{
    (*g_body)();
    g_cur->done = true;
    _longjmp(g_sched_jb, 1);
}

/* kernels of the reference that synchronise their block
 * (src/calculus.h:264,322; src/topological.h:22,486; src/nucleation2.cu:292) */
bool uses_barrier(const char *name)
{
    static const char *k[] = { "grains_per_block", "nucl_area_per_block", "two_three_sided_grains_per_block",
                               "flips_per_block", "get_vertex_id_per_block" };
    for (const char *s : k) if (!strcmp(s, name)) return true;
    return false;
}
} // namespace

void sevc_syncthreads()
{
    if (!g_fiber_mode) { fprintf(stderr, "sevc_ref: __syncthreads outside a barrier kernel\n"); abort(); }
    if (!_setjmp(g_cur->jb)) _longjmp(g_sched_jb, 1);
}

void sevc_launch(const char *name, unsigned int grid, unsigned int block, const std::function<void()> &body)
{
    gridDim = { grid, 1, 1 };
    blockDim = { block, 1, 1 };
    if (!uses_barrier(name)) {
        for (unsigned b = 0; b < grid; b++)
            for (unsigned t = 0; t < block; t++) {
                blockIdx = { b, 0, 0 };
                threadIdx = { t, 0, 0 };
                body();
            }
        return;
    }
    const size_t stack_bytes = 1 << 16;
    if (g_pool.size() < block) {
        g_pool.resize(block);
        for (auto &f : g_pool) if (f.stack.size() < stack_bytes) f.stack.resize(stack_bytes);
    }
    g_fiber_mode = true;
    g_body = &body;
    for (unsigned b = 0; b < grid; b++) {
        blockIdx = { b, 0, 0 };
        for (unsigned t = 0; t < block; t++) {
            Fiber &f = g_pool[t];
            f.done = false;
            f.started = false;
            getcontext(&f.ctx);
            f.ctx.uc_stack.ss_sp = f.stack.data();
            f.ctx.uc_stack.ss_size = f.stack.size();
            f.ctx.uc_link = nullptr;
            makecontext(&f.ctx, fiber_entry, 0);
        }
        bool alive = true;
        while (alive) {
            alive = false;
            for (unsigned t = 0; t < block; t++) {
                Fiber &f = g_pool[t];
                if (f.done) continue;
                threadIdx = { t, 0, 0 };
                g_cur = &f;
                if (!_setjmp(g_sched_jb)) {
                    if (!f.started) { f.started = true; swapcontext(&g_boot, &f.ctx); }
                    else _longjmp(f.jb, 1);
                }
                if (!f.done) alive = true;
            }
        }
    }
    g_fiber_mode = false;
    g_cur = nullptr;
}

/* ---------------- printf guard ---------------- */
int sevc_ref_printf(const char *fmt, ...)
{
    static int quiet = getenv("SEVC_REF_QUIET") != nullptr;
    if (quiet) return 0;
    va_list ap;
    va_start(ap, fmt);
    int r;
    /* src/topological.h:598,601 pass two ints for "In %s: ... (%d and %d)" */
    if (!strncmp(fmt, "In %s: 3 sided grain", 20) || !strncmp(fmt, "In %s: Error: 3 Sided", 21)) {
        int a = va_arg(ap, int), b = va_arg(ap, int);
        r = ::printf("In unlabel_boundaries_st2: (%d and %d) [format guarded]\n", a, b);
    } else {
        r = vprintf(fmt, ap);
    }
    va_end(ap);
    return r;
}

int sevc_ref_min_grains()
{
    const char *s = getenv("SEVC_REF_MIN_GRAINS");
    return s ? atoi(s) : 5000;
}

/* ---------------- random stream ---------------- */
double sevc_ref_rng_draw(long long tid, long long pos)
{
    static bool init = false;
    static uint64_t seed = 0;
    static std::vector<double> table;
    static long long ndraws = 0;
    if (!init) {
        init = true;
        if (const char *s = getenv("SEVC_REF_RNG_SEED")) seed = strtoull(s, nullptr, 10);
        if (const char *p = getenv("SEVC_REF_RNG_TABLE")) {
            ndraws = atoll(getenv("SEVC_REF_RNG_NDRAWS") ? getenv("SEVC_REF_RNG_NDRAWS") : "0");
            FILE *f = fopen(p, "rb");
            if (!f || ndraws <= 0) { fprintf(stderr, "sevc_ref: bad rng table\n"); exit(3); }
            fseek(f, 0, SEEK_END);
            long n = ftell(f) / (long)sizeof(double);
            fseek(f, 0, SEEK_SET);
            table.resize((size_t)n);
            if (fread(table.data(), sizeof(double), (size_t)n, f) != (size_t)n) exit(3);
            fclose(f);
        }
    }
    if (!table.empty()) {
        if (pos >= ndraws) { fprintf(stderr, "sevc_ref: rng table exhausted (stream %lld)\n", tid); exit(3); }
        return table[(size_t)(tid * ndraws + pos)];
    }
    return sevc_synth_uniform(seed, (uint64_t)tid, (uint64_t)pos);
}

int main(int argc, char const *argv[])
{
    setvbuf(stdout, nullptr, _IOFBF, 1 << 20);
    return sevc_ref_main(argc, argv);
}
