// jt_pow2_f64.cu -- instantiations of the register-resident power-of-two
// Stockham kernel (jt_stockham.cuh) for double.
#include "jt_stockham.cuh"

namespace jt {

// Launches the kernel for line length L; returns false when (L, mode) has no
// instantiation (row mode: 16..8192, column modes: 16..4096).
bool stockham_launch(int L, int mode, int sign, const V2<double>::t *in, V2<double>::t *out, const StockParams &p,
                     const V2<double>::t *W, const V2<double>::t *Whi, const V2<double>::t *Wlo, cudaStream_t s) {
#define JT_CASE(LL)                                                         \
    case LL:                                                                \
        StockLaunch<double, LL>::go(mode, sign, in, out, p, W, Whi, Wlo, s);  \
        return true;
    if (mode == 0) {
        switch (L) {
            JT_CASE(16) JT_CASE(32) JT_CASE(64) JT_CASE(128) JT_CASE(256) JT_CASE(512) JT_CASE(1024)
            JT_CASE(2048) JT_CASE(4096) JT_CASE(8192)

            default: return false;
        }
    }
    switch (L) {
        JT_CASE(16) JT_CASE(32) JT_CASE(64) JT_CASE(128) JT_CASE(256) JT_CASE(512) JT_CASE(1024)
        JT_CASE(2048) JT_CASE(4096)
        default: return false;
    }
#undef JT_CASE
}

int stockham_lines_per_cta(int L, int mode, const double *) { return StockCfg<double>::C(L, mode); }

}  // namespace jt
