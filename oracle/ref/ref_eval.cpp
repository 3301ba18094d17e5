// Reference evaluation-tool harness: the reference's own shared/tools/eval_tools.cpp compiled
// against oracle/ref_shim with its CLI main() renamed away.
//
// TEST INFRASTRUCTURE ONLY. Built into oracle/_ref/ by oracle/Makefile; used by the tests to
// pin the C restatement of the metrics (oracle/rpd_oracle.c orc_hdr_metrics) and to produce
// the metrics golden vectors.
#define main rpd_reference_eval_cli_main
#include "shared/tools/eval_tools.cpp"
#undef main

#include <unistd.h>

#include <cstdio>
#include <string>

namespace {
void put(const char* name, const float* data, int w, int h) {
    stb_shim::Img img;
    img.w = w;
    img.h = h;
    img.comp = 3;
    img.data.assign(data, data + size_t(w) * h * 3);
    stb_shim::table()[name] = img;
}
}  // namespace

extern "C" {

// compute_extended_metrics (eval_tools.cpp:121-213): out = {nrmse, log_ssim11, log_gradient_nrmse}.
void ref_extended_metrics(const float* ref, const float* tst, int w, int h, double* out) {
    const ExtendedMetrics m = compute_extended_metrics(ref, tst, w, h);
    out[0] = m.nrmse;
    out[1] = m.log_ssim11;
    out[2] = m.log_gradient_nrmse;
}

// `eval_tools hdr-metrics ref tst` on in-memory images; its report (stdout) into buf.
int ref_hdr_metrics_text(const float* ref, const float* tst, int w, int h, char* buf, int cap) {
    put("ref", ref, w, h);
    put("tst", tst, w, h);
    std::fflush(stdout);
    int fds[2];
    if (pipe(fds) != 0) return -1;
    const int saved = dup(1);
    dup2(fds[1], 1);
    char a0[] = "eval_tools", a1[] = "hdr-metrics", a2[] = "ref", a3[] = "tst";
    char* argv[] = {a0, a1, a2, a3, nullptr};
    const int rc = rpd_reference_eval_cli_main(4, argv);
    std::fflush(stdout);
    dup2(saved, 1);
    close(saved);
    close(fds[1]);
    const ssize_t n = read(fds[0], buf, size_t(cap - 1));
    close(fds[0]);
    buf[n > 0 ? n : 0] = '\0';
    return rc;
}

}  // extern "C"
