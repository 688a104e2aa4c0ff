// gputracetask.h -- the reference-side render task of the drop-in boundary:
// a RenderTask that drains the view's render blocks like TraceTask does
// (source/backend/render/tracetask.cpp:287-454) and traces them through
// libpovgpu's C ABI (include/povgpu.h), compiled against the reference's
// RenderTask / ViewData headers.  View::StartRender would create one of
// these instead of its +WT TraceTasks (source/backend/scene/view.cpp:
// 1141-1190) when the GPU option is set, after flattening SceneData once
// (pov_flatten.h) into the PovGpuScene handed in here.
#ifndef POV_GPUTRACETASK_H
#define POV_GPUTRACETASK_H

#include "backend/render/rendertask.h"

#include "povgpu.h"

namespace pov {

class GpuTraceTask final : public RenderTask
{
    public:
        // `scene` is owned by the caller (one per View); `batch` bounds the
        // blocks traced per library call so Cooperate() runs between calls.
        GpuTraceTask(ViewData *vd, PovGpuScene *scene, const PovGpuRenderParams& params, size_t batch = 4096);
        virtual ~GpuTraceTask() override;

        virtual void Run() override;
        virtual void Stopped() override;
        virtual void Finish() override;
    private:
        PovGpuScene *mScene;
        PovGpuRenderParams mParams;
        size_t mBatch;
};

}

#endif
