// ref_qef.cpp -- the reference's own QEF solve (leven/cl/qef.cl), compiled on
// the host through cl_shim.h, behind a C entry point.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/Makefile into oracle/_ref where
// the reference tree is present, and used only by tests to pin the oracle's
// restatement of qef_add_point / qef_solve.  Compiled with -ffp-contract=off
// (no multiply-add is fused outside dot(), the restatement's convention for
// the QEF) and -fsingle-precision-constant (qef.cl's double literals, as in
// `2.0 * c * s * a` and `1.0 / x`, are single precision).
#include "cl_shim.h"

#define constant static const

#include "cl/qef.cl"

extern "C" {

// qef_create_from_points (qef.cl:283-303) over `count` points and normals
// (x, y, z, w each), then qef_solve (qef.cl:239-256).  out: the solved
// position (x, y, z, w); returns qef_solve's error.
float ref_qef_solve_points(const float* positions, const float* normals, int count, float* out) {
    float4 p[12], n[12];
    for (int i = 0; i < count && i < 12; i++) {
        p[i] = float4(positions[4 * i], positions[4 * i + 1], positions[4 * i + 2], positions[4 * i + 3]);
        n[i] = float4(normals[4 * i], normals[4 * i + 1], normals[4 * i + 2], normals[4 * i + 3]);
    }
    QEFData q;
    qef_create_from_points(p, n, (size_t)(count < 12 ? count : 12), &q);
    float4 x = {0.f, 0.f, 0.f, 0.f};
    const float err = qef_solve(&q, &x);
    out[0] = x.x;
    out[1] = x.y;
    out[2] = x.z;
    out[3] = x.w;
    return err;
}

}
