// bem: the command-line program of main.rs:1-9 over libbem_gb300.so.
//
//   bem input.json
//
// reads the input file (analysis.rs:42-48 input_from_file), runs every
// frequency in the plain FP64 form (analysis.rs:57-118 run, results converted
// as postprocess.rs:70-79 leaves them) and writes the results at the first
// frequency to the input's output.file (analysis.rs:121-123
// write_results_at_frequency(0)).  Where the reference panics, this prints
// the library's message and exits with status 1.
#include <cstdio>
#include <vector>

#include "bem.h"

static int fail(bem_ctx* ctx, const char* what, bem_status st) {
    std::fprintf(stderr, "bem: %s failed (status %d): %s\n", what, (int)st, ctx ? bem_last_error(ctx) : "");
    return 1;
}

int main(int argc, char** argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: bem <input.json>\n");
        return 1;
    }
    std::printf(" Attempting to read input file: %s\n", argv[1]);
    bem_ctx* ctx = nullptr;
    bem_status st = bem_ctx_create(0, &ctx);
    if (st != BEM_OK) return fail(nullptr, "creating the GPU context", st);
    bem_problem* p = nullptr;
    if ((st = bem_problem_from_file(ctx, argv[1], &p)) != BEM_OK) return fail(ctx, "reading the input", st);
    bem_problem_info info;
    bem_problem_get_info(p, &info);
    const size_t nfp = (size_t)info.num_field_points, nf = (size_t)info.num_frequencies;
    const size_t total = (size_t)info.num_rhs * nf * nfp;
    std::vector<bem_cplx> scattered(total > 0 ? total : 1), incident(total > 0 ? total : 1);
    if ((st = bem_run(ctx, p, BEM_FORM_PLAIN_FP64, BEM_PRECOND_NONE, scattered.data(), incident.data(), nullptr, 0)) !=
        BEM_OK)
        return fail(ctx, "the analysis", st);
    if ((st = bem_write_results_at_frequency(ctx, p, nullptr, scattered.data(), incident.data())) != BEM_OK)
        return fail(ctx, "writing the results", st);
    std::printf(" Complete!\n");
    bem_problem_destroy(p);
    bem_ctx_destroy(ctx);
    return 0;
}
