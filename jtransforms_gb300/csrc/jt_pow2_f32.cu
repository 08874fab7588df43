// jt_pow2_f32.cu -- instantiations of the register-resident power-of-two
// Stockham kernels (jt_stockham.cuh) for float.
#include "jt_stockham.cuh"

namespace jt {

// Whether the pipelined (TMA) kernel exists for (L, mode).
bool stockham_pipe_ok(int L, int mode, const float *) {
#define JT_PCASE(LL) \
    case LL:         \
        return mode == 0 ? (Stockham<float, LL, 0, -1>::PIPE_OK || Stockham<float, LL, 0, -1>::BIG_OK) : (LL <= 4096 && Stockham<float, (LL <= 4096 ? LL : 16), 1, -1>::PIPE_OK);
    switch (L) {
        JT_PCASE(16) JT_PCASE(32) JT_PCASE(64) JT_PCASE(128) JT_PCASE(256) JT_PCASE(512) JT_PCASE(1024)
        JT_PCASE(2048) JT_PCASE(4096) JT_PCASE(8192)
        JT_PCASE(16384)
        default: return false;
    }
#undef JT_PCASE
}

// Lines per CTA of (L, mode).
int stockham_lines_per_cta(int L, int mode, const float *) { return StockCfg<float>::C(L, mode); }

// Launches the kernel for line length L; returns false when (L, mode) has no
// instantiation (row mode: 16..16384, column modes: 16..4096).  A non-null
// `tmap` selects the pipelined TMA kernel (the caller has checked
// stockham_pipe_ok and the 16-byte rules).
bool stockham_launch(int L, int mode, int sign, const V2<float>::t *in, V2<float>::t *out, const StockParams &p,
                     const CUtensorMap *tmap, const V2<float>::t *W, const V2<float>::t *Whi, const V2<float>::t *Wlo,
                     int *err, int sms, cudaStream_t s) {
#define JT_CASE(LL)                                                                       \
    case LL:                                                                              \
        StockLaunch<float, LL>::go(mode, sign, in, out, p, tmap, W, Whi, Wlo, err, sms, s); \
        return true;
    if (mode == 0) {
        switch (L) {
            JT_CASE(16) JT_CASE(32) JT_CASE(64) JT_CASE(128) JT_CASE(256) JT_CASE(512) JT_CASE(1024)
            JT_CASE(2048) JT_CASE(4096) JT_CASE(8192)
            JT_CASE(16384)
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

}  // namespace jt
