// Device helpers shared by the window kernels of all models: the driver-table cursor.
#pragma once

#include <cuda_runtime.h>

#include "../../include/lfdm/device/fp_order.cuh"

namespace lfdm {

constexpr int kMaxSmemClasses = 8;

struct DriverCursor {
    const double* rows;
    int len;
    int r;  // first row with time >= t (valid while rows[0].t < t < rows[len-1].t)
    long long kfirst, klast;  // order keys of the first and last row times
};

__device__ __forceinline__ void driver_begin(DriverCursor& c, const double* rows, int len, double t) {
    c.rows = rows;
    c.len = len;
    c.kfirst = okey(__ldg(rows));
    c.klast = okey(__ldg(rows + 4 * (len - 1)));
    int l = 0, h = len;
    while (l < h) {
        int mid = (l + h) >> 1;
        if (t <= __ldg(rows + 4 * mid)) h = mid;
        else l = mid + 1;
    }
    c.r = l;
}

// GetDriverInput (utils/utils_gpu.cu:34-56) with a monotone cursor in place of the per-step
// binary search; the segment found is the same lower_bound segment for non-decreasing tables. The
// time tests compare order keys (integer pipe), with the results of the floating-point tests.
__device__ __forceinline__ void driver_at(DriverCursor& c, double t, double& st, double& th, double& br) {
    const long long kt = okey(t);
    if (kt <= c.kfirst) {
        st = __ldg(c.rows + 1);
        th = __ldg(c.rows + 2);
        br = __ldg(c.rows + 3);
        return;
    }
    if (kt >= c.klast) {
        const double* L = c.rows + 4 * (c.len - 1);
        st = __ldg(L + 1);
        th = __ldg(L + 2);
        br = __ldg(L + 3);
        return;
    }
    while (okey(__ldg(c.rows + 4 * c.r)) < kt) ++c.r;
    while (c.r > 1 && okey(__ldg(c.rows + 4 * (c.r - 1))) >= kt) --c.r;  // t moved backwards (new window)
    const double2* L = reinterpret_cast<const double2*>(c.rows + 4 * (c.r - 1));
    const double2 L01 = __ldg(L), L23 = __ldg(L + 1), R01 = __ldg(L + 2), R23 = __ldg(L + 3);
    const double tbar = (t - L01.x) / (R01.x - L01.x);
    st = L01.y + tbar * (R01.y - L01.y);
    th = L23.x + tbar * (R23.x - L23.x);
    br = L23.y + tbar * (R23.y - L23.y);
}

}  // namespace lfdm
