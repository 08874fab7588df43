// jt_r2r_f32.cu -- instantiations of the register-form DCT/DST/DHT line
// kernels (jt_r2r.cuh) for float, half lengths 16..4096.
#include "jt_r2r.cuh"

namespace jt {

// Rows (lines) per CTA of the register form for half length H; 0 when H has none.
int r2r_reg_lines(int H, const float *) {
    switch (H) {
        case 16: return Stockham<float, 16, 0, -1>::C;
        case 32: return Stockham<float, 32, 0, -1>::C;
        case 64: return Stockham<float, 64, 0, -1>::C;
        case 128: return Stockham<float, 128, 0, -1>::C;
        case 256: return Stockham<float, 256, 0, -1>::C;
        case 512: return Stockham<float, 512, 0, -1>::C;
        case 1024: return Stockham<float, 1024, 0, -1>::C;
        case 2048: return Stockham<float, 2048, 0, -1>::C;
        case 4096: return Stockham<float, 4096, 0, -1>::C;
        default: return 0;
    }
}

bool r2r_reg_launch(int H, int op, const float *in, float *out, const R2rParams &p, const V2<float>::t *Wp,
                    const V2<float>::t *Wr, const V2<float>::t *Wd, cudaStream_t s) {
#define JT_RCASE(HH)                                                       \
    case HH:                                                               \
        R2rRegLaunch<float, HH>::go(op, in, out, p, Wp, Wr, Wd, s);          \
        return true;
    switch (H) {
        JT_RCASE(16) JT_RCASE(32) JT_RCASE(64) JT_RCASE(128) JT_RCASE(256) JT_RCASE(512) JT_RCASE(1024) JT_RCASE(2048)
        JT_RCASE(4096)
        default: return false;
    }
#undef JT_RCASE
}

}  // namespace jt
