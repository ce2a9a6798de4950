// pb_batch.cu -- batched solves of independent problems (local bundle-adjustment windows).
//
// The reference solves one problem per Solver::solve call; a caller with many local windows
// calls it once per window.  pb_gpu_solve_batch keeps the per-problem semantics (each problem is
// solved exactly as pb_gpu_solve_problem solves it) and gets the windows onto the device
// together: n_workers host threads each own a context with its own stream and take problems from
// a shared queue, so the kernels of different windows overlap on the GPU, their host-side
// planning overlaps on the CPU (each worker's planning threads capped at the host cores divided
// by the workers), and a context's device memory is reused from one window to the next (slab
// arena).  The cooperative solvers size their grids to the window.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <thread>
#include <vector>

#include "pb_internal.h"

extern "C" pb_status pb_gpu_solve_batch(int32_t device, int32_t n_problems, const pb_problem_desc* problems,
                                        const pb_solve_options* options, int32_t n_workers, pb_solve_report* reports,
                                        double* const* cameras_out, double* const* points_out,
                                        int8_t* const* valid_out, double* latency_ms) {
    if (n_problems < 0 || (n_problems > 0 && (!problems || !options || !reports))) return PB_ERR_INVALID_ARGUMENT;
    if (n_workers <= 0) return PB_ERR_INVALID_ARGUMENT;
    if (n_problems == 0) return PB_OK;
    const int workers = std::min<int>(n_workers, n_problems);
    std::atomic<int> next{0};
    std::atomic<int> first_error{PB_OK};
    auto note = [&](pb_status st) {
        int expected = PB_OK;
        if (st != PB_OK) first_error.compare_exchange_strong(expected, st);
    };
    // the workers share the host cores for their planning (the plan does not depend on it)
    const int cap = std::max(1, static_cast<int>(std::max(1u, std::thread::hardware_concurrency())) / workers);
    auto work = [&]() {
        pb::set_host_thread_cap(cap);
        pb_gpu_ctx* ctx = nullptr;
        const pb_status cs = pb_gpu_create(device, &ctx);
        if (cs != PB_OK) {
            note(cs);
            pb::set_host_thread_cap(0);
            return;
        }
        for (int i = next.fetch_add(1); i < n_problems; i = next.fetch_add(1)) {
            const auto t0 = std::chrono::steady_clock::now();
            const pb_status st = pb_gpu_solve_problem(ctx, &problems[i], options, &reports[i],
                                                      cameras_out ? cameras_out[i] : nullptr,
                                                      points_out ? points_out[i] : nullptr,
                                                      valid_out ? valid_out[i] : nullptr, nullptr, nullptr);
            if (latency_ms)
                latency_ms[i] = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
            note(st);
        }
        pb_gpu_destroy(ctx);
        pb::set_host_thread_cap(0);
    };
    std::vector<std::thread> pool;
    pool.reserve(workers - 1);
    for (int w = 1; w < workers; ++w) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    return static_cast<pb_status>(first_error.load());
}
