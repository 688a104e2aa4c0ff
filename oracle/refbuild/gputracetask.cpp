// gputracetask.cpp -- see gputracetask.h.
#include "gputracetask.h"

#include <vector>

#include "base/types.h"
#include "core/support/statistics.h"
#include "backend/scene/view.h"
#include "backend/scene/viewthreaddata.h"

namespace pov {

GpuTraceTask::GpuTraceTask(ViewData *vd, PovGpuScene *scene, const PovGpuRenderParams& params, size_t batch) :
    RenderTask(vd, 0, "GpuTrace"), mScene(scene), mParams(params), mBatch(batch > 0 ? batch : 1)
{}

GpuTraceTask::~GpuTraceTask() {}

// TraceTask::Run's block loop: GetNextRectangle hands out the blocks
// (ViewData::GetNextRectangle, view.cpp:236, skipping the blocks a
// continued trace already has), each batch is traced in one library call,
// and each block's pixels go back through CompletedRectangle
// (view.cpp:405) exactly as TraceTask returns them: the rectangle's RGBT
// row by row.  The library's counters are added to the view's statistics
// under the reference's own names.
void GpuTraceTask::Run()
{
    for (;;)
    {
        std::vector<PovGpuBlock> blocks;
        std::vector<POVRect> rects;
        std::vector<unsigned int> serials;
        POVRect rect;
        unsigned int serial;
        while (blocks.size() < mBatch && GetViewData()->GetNextRectangle(rect, serial))
        {
            PovGpuBlock b = {};
            b.left = (int32_t)rect.left;
            b.top = (int32_t)rect.top;
            b.right = (int32_t)rect.right;
            b.bottom = (int32_t)rect.bottom;
            b.serial = serial;
            blocks.push_back(b);
            rects.push_back(rect);
            serials.push_back(serial);
        }
        if (blocks.empty())
            break;
        size_t npix = 0;
        for (const POVRect& r : rects)
            npix += r.GetArea();
        std::vector<float> rgbt(npix * 4);
        PovGpuStats st = {};
        const int rc = pov_gpu_trace_blocks(mScene, blocks.data(), (int32_t)blocks.size(), &mParams,
                                            rgbt.data(), &st);
        if (rc != POV_GPU_OK)
            throw POV_EXCEPTION_STRING(pov_gpu_error_string(rc));
        size_t off = 0;
        for (size_t b = 0; b < rects.size(); b++)
        {
            std::vector<RGBTColour> pixels(rects[b].GetArea());
            for (size_t k = 0; k < pixels.size(); k++, off++)
                pixels[k] = RGBTColour(rgbt[4 * off], rgbt[4 * off + 1], rgbt[4 * off + 2], rgbt[4 * off + 3]);
            GetViewData()->CompletedRectangle(rects[b], serials[b], pixels, 1, true, true);
        }
        RenderStatistics& stats = GetViewDataPtr()->Stats();
        stats[Number_Of_Pixels] += st.number_of_pixels;
        stats[Number_Of_Samples] += st.number_of_samples;
        stats[Number_Of_Rays] += st.number_of_rays;
        stats[Shadow_Ray_Tests] += st.shadow_ray_tests;
        stats[Shadow_Rays_Succeeded] += st.shadow_rays_succeeded;
        stats[Reflected_Rays_Traced] += st.reflected_rays;
        stats[Transmitted_Rays_Traced] += st.transmitted_rays;
        stats[Refracted_Rays_Traced] += st.refracted_rays;
        stats[Internal_Reflected_Rays_Traced] += st.internal_reflected_rays;
        stats[Media_Samples] += st.media_samples;
        Cooperate();   // stop / pause between library calls
    }
}

void GpuTraceTask::Stopped() {}

void GpuTraceTask::Finish()
{
    GetViewDataPtr()->timeType = TraceThreadData::kRenderTime;
    GetViewDataPtr()->realTime = ConsumedRealTime();
    GetViewDataPtr()->cpuTime = ConsumedCPUTime();
}

}
