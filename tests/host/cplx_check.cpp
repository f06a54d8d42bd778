// Host check of the complex-step type used by the GPU's complex build:
// reads "x y" pairs on stdin, prints sqrt_, acos_, sin_, cos_ of x + i y and
// of the quotient (x + i y) / (y + i x) as re/im pairs, one line per input.
#include <cstdio>

#include "idw_cplx.cuh"

using idw::cplx;

int main() {
    double x, y;
    while (std::scanf("%lf %lf", &x, &y) == 2) {
        const cplx z(x, y);
        const cplx r[5] = {idw::sqrt_(z), idw::acos_(z), idw::sin_(z), idw::cos_(z), z / cplx(y, x)};
        for (const cplx &v : r) std::printf("%.17g %.17g ", v.re, v.im);
        std::printf("\n");
    }
    return 0;
}
