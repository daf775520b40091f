// Dense GMRES without any device allocation: the solver's working memory is a
// fixed-size array that lives in the library's device image, so a call only
// launches kernels and copies a few bytes.  This serves callers that cannot
// allocate device memory at solve time: applications that hand all device
// memory to their own pool up front (a framework's caching allocator, a
// real-time loop with a fixed memory budget) and would otherwise see a
// cudaMalloc that synchronises the device or fails under their budget.
#include <chrono>
#include <cmath>
#include <mutex>

#include "common.cuh"
#include "gmres.cuh"

namespace bem {

// Scratch capacity: n up to 4096 for every iteration limit (larger n fit when
// max_iterations keeps the restart length small).  Every GPU that loads the
// library holds this array until the process exits.
constexpr size_t NOALLOC_SCRATCH_BYTES = 8u << 20;

// In host code this name is only a stand-in for the device symbol: its device
// address comes from cudaGetSymbolAddress below and is what the kernels get.
static __device__ __align__(256) unsigned char g_gmres_scratch[NOALLOC_SCRATCH_BYTES];

namespace {
constexpr int MAX_DEVICES = 64;
std::mutex g_setup_mutex;
void* g_scratch_ptr[MAX_DEVICES] = {};

// Once per device, with that device current: resolve the array's device
// address.  The address is kept for the life of the process, so the entry
// point is not valid after cudaDeviceReset (or any other re-creation of the
// device's primary context) in the same process.
void* scratch_address(int device) {
    require(device >= 0 && device < MAX_DEVICES, "device index out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_gmres_scratch);
        if (e != cudaSuccess || !p)
            throw Error(BEM_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
        g_scratch_ptr[device] = p;
    }
    return g_scratch_ptr[device];
}
}  // namespace

}  // namespace bem

using namespace bem;

extern "C" {

BEM_API bem_status bem_gmres_solve_noalloc(bem_ctx* ctx, int64_t n, const bem_cplx* A, int64_t lda, int64_t max_it,
                                           double tol, bem_cplx* x, bem_solve_report* report) {
    if (!ctx || !A || !x || n <= 0 || lda < n) return BEM_ERR_BAD_INPUT;
    if (report) {
        *report = bem_solve_report{};
        report->rel_err_vs_lu = -1;
    }
    Context& c = ctx->c;
    const auto t0 = std::chrono::steady_clock::now();
    try {
        BEM_CUDA(cudaSetDevice(c.device));
        // the restart rule of gmres.rs:41-48
        if (max_it <= 0) max_it = 1000;
        if (max_it > n) max_it = n;
        if (tol <= 0.0) tol = 1e-5;
        const int m = (int)std::ceil(std::sqrt((double)max_it));
        const int64_t restarts = max_it / m;
        void* scratch = scratch_address(c.device);
        GmWorkspace ws;
        const size_t need = gm_prepare_external(c, ws, 1, n, m, A, lda, 0, false, true, scratch,
                                                NOALLOC_SCRATCH_BYTES);
        require(need <= NOALLOC_SCRATCH_BYTES,
                "bem_gmres_solve_noalloc: n = " + std::to_string(n) + " with restart length " + std::to_string(m) +
                    " needs " + std::to_string(need) + " bytes of scratch; the fixed scratch holds " +
                    std::to_string(NOALLOC_SCRATCH_BYTES) + " bytes (n up to 4096 at any iteration limit)");
        BEM_CUDA(cudaMemcpyAsync(ws.bt.B, x, sizeof(double2) * n, cudaMemcpyDeviceToDevice, c.stream));
        gm_matrix_norms(c, ws);
        gm_init(c, ws, tol, restarts);
        GmState st{};
        const int64_t limit = restarts * (int64_t)m + 1;
        for (int64_t it = 0; it < limit; ++it) {
            gm_launch_iteration(c, ws, nullptr, nullptr);
            BEM_CUDA(cudaMemcpyAsync(&st, ws.bt.st, sizeof(GmState), cudaMemcpyDeviceToHost, c.stream));
            BEM_CUDA(cudaStreamSynchronize(c.stream));
            if (st.done) break;
        }
        BEM_CUDA(cudaMemcpyAsync(x, ws.bt.X, sizeof(double2) * n, cudaMemcpyDeviceToDevice, c.stream));
        BEM_CUDA(cudaStreamSynchronize(c.stream));
        if (report) {
            report->num_mv = st.num_mv;
            report->restarts = st.restarts + (st.converged ? 1 : 0);
            report->iterations = st.iterations;
            report->backward_error = st.error;
            report->flag = st.converged ? 1 : 2;
            report->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        }
        return st.converged ? BEM_OK : BEM_ERR_NOT_CONVERGED;
    } catch (const Error& e) {
        c.last_error = e.what();
        return e.status;
    } catch (const std::exception& e) {
        c.last_error = e.what();
        return BEM_ERR_CUDA;
    }
}

}  // extern "C"
