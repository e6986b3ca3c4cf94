// Host build of the double-float arithmetic (etraj.jl_gb300/csrc/dfloat.h) for
// tests/test_dfloat.py: each entry point applies one operation elementwise to
// double-float inputs given as (hi, lo) float pairs and returns pairs.
#include "dfloat.h"

using etraj::df;

extern "C" {

void probe_op(int op, long n, const float* a, const float* b, float* out) {
    for (long i = 0; i < n; ++i) {
        const df x{a[2 * i], a[2 * i + 1]}, y{b[2 * i], b[2 * i + 1]};
        df r{0.0f, 0.0f};
        switch (op) {
            case 0: r = etraj::df_add(x, y); break;
            case 1: r = etraj::df_mul(x, y); break;
            case 2: r = etraj::df_div(x, y); break;
            case 3: r = etraj::df_sqrt(x); break;
            case 4: r = etraj::df_rsqrt(x); break;
            case 5: r = etraj::df_exp_neg(x, etraj::kExp2Tab); break;
            case 6: r = etraj::df_fma(x, y, x); break;
            case 7: r = etraj::df_sqr(x); break;
            case 8: r = etraj::df_rcp(x); break;
            case 9: r = etraj::df_exp2(x, etraj::kExp2Tab); break;
            case 10: r = etraj::df_log2(x, etraj::kLog2cTab, etraj::kRcpcTab); break;
            default: break;
        }
        out[2 * i] = r.hi;
        out[2 * i + 1] = r.lo;
    }
}

void probe_exp2_table(float* out) {
    for (int i = 0; i < 2 * etraj::kExpTabN; ++i) out[i] = etraj::kExp2Tab[i];
}
}
