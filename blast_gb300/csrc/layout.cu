// Batched copies between matrix layouts (dense column-major, row-major, panel), binary64.
//
// Reference: BLAST's assign() between panel and dense matrices (expressions/PanelMatrix.hpp:63-240)
// and its panel addressing (panel/StaticPanelMatrix.hpp:178-184). One warp per instance; lanes
// walk the destination in its own storage order so that the stores are coalesced for dense and
// panel destinations alike (a panel of height ps stores ps consecutive rows of each column).
#include "common.cuh"

namespace blastgpu {
namespace {

__global__ void __launch_bounds__(128) copy_kernel(const blastgpu_copy_desc* desc, int64_t count, int32_t* status) {
    int64_t const b = (int64_t)blockIdx.x * 4 + (threadIdx.x >> 5);
    int const lane = threadIdx.x & 31;
    if (b >= count) return;
    blastgpu_copy_desc const d = desc[b];
    if (d.src.rows != d.dst.rows || d.src.cols != d.dst.cols) {
        if (status && lane == 0) status[b] = -1;
        return;
    }
    MatView const s = view(d.src), t = view(d.dst);
    int const m = d.dst.rows, n = d.dst.cols;
    bool const row_major = d.dst.layout == BLASTGPU_ROW_MAJOR;
    // a panel destination is walked slot by slot, padding rows of the last panel included
    int64_t const total = d.dst.layout == BLASTGPU_PANEL
                              ? (int64_t)((m + t.ps - 1) / t.ps) * t.ps * n
                              : (int64_t)m * n;
    for (int64_t e = lane; e < total; e += 32) {
        int i, j;
        if (row_major) { i = (int)(e / n); j = (int)(e % n); }
        else if (d.dst.layout == BLASTGPU_PANEL) {
            // walk panel by panel, column by column inside a panel
            int const ps = t.ps, per_panel = ps * n;
            int const p = (int)(e / per_panel), w = (int)(e % per_panel);
            j = w / ps;
            i = p * ps + w % ps;
            if (i >= m) continue;
        } else { i = (int)(e % m); j = (int)(e / m); }
        t(i, j) = s(i, j);
    }
    if (status && lane == 0) status[b] = 0;
}

}  // namespace
}  // namespace blastgpu

using namespace blastgpu;

extern "C" {

int blastgpu_dcopy_batched(const blastgpu_copy_desc* desc, int64_t batch, int32_t* status,
                           blastgpu_stream_t stream) {
    if (batch < 0) return -2;
    if (batch == 0) return BLASTGPU_SUCCESS;
    if (!desc) return -1;
    int64_t const blocks = (batch + 3) / 4;
    if (blocks > 0x7fffffff) return BLASTGPU_ERR_TOO_LARGE;
    copy_kernel<<<(unsigned)blocks, 128, 0, as_cuda(stream)>>>(desc, batch, status);
    return check_launch();
}

}  // extern "C"
