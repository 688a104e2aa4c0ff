// pov_oracle -- per-ray / per-pixel dump harness around the reference
// renderer, built from the unmodified reference sources (oracle/refbuild/
// Makefile).  Test infrastructure only: it produces the golden vectors that
// pin the oracle restatement and the GPU path.
//
// It does what the reference's own tasks do for one view, without the
// POVMS front end:
//   ParserTask::Run          (source/backend/control/parsertask.cpp)
//   BoundingTask::Run        (source/backend/bounding/boundingtask.cpp:168)
//   TraceTask / TracePixel   (source/backend/render/tracetask.cpp:403,
//                             source/core/render/tracepixel.cpp:311)
//   Trace::FindIntersection  (source/core/render/trace.cpp:230)
//
// Usage:
//   pov_oracle SCENE.pov W H pixels OUT.rgbt        float32 RGBT, row-major
//   pov_oracle SCENE.pov W H rays   IN.rays OUT.hits
//        IN.rays:  int32 n, then n * (origin[3], dir[3]) doubles
//        OUT.hits: n * (int32 object, int32 triangle, double depth)
//   pov_oracle SCENE.pov W H scene  OUT.txt          parsed camera + objects
//   pov_oracle SCENE.pov W H desc   OUT.pgsf         the parsed scene flattened
//        into the C ABI's scene description (pov_flatten.cpp), as a scene file
// Every mode prints one JSON line of render statistics on stdout.

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <string>
#include <vector>
#include <execinfo.h>
#include <csignal>
#include <unistd.h>

#include "base/fileinputoutput.h"
#include "base/messenger.h"
#include "base/platformbase.h"
#include "base/stringutilities.h"
#include "core/bounding/boundingbox.h"
#include "core/lighting/lightsource.h"
#include "core/material/media.h"
#include "core/material/noise.h"
#include "core/material/pattern.h"
#include "core/math/matrix.h"
#include "core/math/randomsequence.h"
#include "core/render/ray.h"
#include "core/render/trace.h"
#include "core/render/tracepixel.h"
#include "core/scene/object.h"
#include "core/scene/scenedata.h"
#include "core/scene/tracethreaddata.h"
#include "core/shape/csg.h"
#include "core/shape/mesh.h"
#include "core/support/statistics.h"
#include "parser/parser.h"

#include "pov_flatten.h"

using namespace pov;
using namespace pov_base;
using namespace pov_parser;

namespace {

struct HarnessSceneData final : public SceneData
{
    HarnessSceneData() : SceneData() {}
};

class HarnessMessenger final : public GenericMessenger
{
public:
    HarnessMessenger() : GenericMessenger(0, "pov_oracle") {}
protected:
    virtual void SendMessage(MessageClass mc, WarningLevel level, const char *text,
                             const UCS2String& filename = u"", POV_LONG line = -1,
                             POV_LONG column = -1, POV_OFF_T offset = -1) override
    {
        if (mc == kMessageClass_Error || mc == kMessageClass_PossibleError)
            std::fprintf(stderr, "pov_oracle: %s\n", text);
    }
};

class HarnessFiles final : public FileResolver, public ProgressReporter
{
public:
    virtual UCS2String FindFile(UCS2String parsedFileName, unsigned int) override
    {
        return parsedFileName;
    }
    virtual IStream* ReadFile(const UCS2String&, const UCS2String& foundFileName, unsigned int) override
    {
        IStream *s = new IFileStream(foundFileName);
        if (!*s)
        {
            delete s;
            return nullptr;
        }
        return s;
    }
    virtual OStream* CreateFile(const UCS2String&, unsigned int, bool) override { return nullptr; }
    virtual void ReportProgress(POV_LONG) override {}
};

// Object ids: SceneData::objects in order (light sources skipped), CSG
// children depth-first right after their parent.
void NumberObjects(ObjectPtr o, std::map<ConstObjectPtr, int>& ids, std::vector<ObjectPtr>& flat)
{
    ids[o] = (int)flat.size();
    flat.push_back(o);
    if (o->Type & IS_COMPOUND_OBJECT)
    {
        CompoundObject *c = dynamic_cast<CompoundObject *>(o);
        if (c != nullptr && !(o->Type & LIGHT_SOURCE_OBJECT))
            for (ObjectPtr ch : c->children)
                NumberObjects(ch, ids, flat);
    }
}

struct Harness
{
    std::shared_ptr<SceneData> sd;
    std::map<ConstObjectPtr, int> ids;
    std::vector<ObjectPtr> flat;

    void Parse(const char *file, double width, double height)
    {
        sd = std::make_shared<HarnessSceneData>();
        sd->inputFile = ASCIItoUCS2String(file);
        sd->headerFile = UCS2String();
        sd->aspectRatio = width / height;
        sd->boundingMethod = 1;
        sd->outputAlpha = false;
        sd->backgroundColour.Clear();
        HarnessMessenger messenger;
        HarnessFiles files;
        TraceThreadData parseData(sd, 0);
        if (std::getenv("POV_ORACLE_DEBUG")) std::fprintf(stderr, "parse start\n");
        {
            Parser parser(sd, ParserOptions(false, 0.0, 0), messenger, files, files, parseData);
            parser.Run();
            if (std::getenv("POV_ORACLE_DEBUG")) std::fprintf(stderr, "parse done\n");
            parser.Finish();
        }
        if (std::getenv("POV_ORACLE_DEBUG")) std::fprintf(stderr, "objects %zu\n", sd->objects.size());
        // BoundingTask::Run with the default threshold of 3 objects.
        if (sd->objects.size() < 3)
        {
            sd->boundingMethod = 0;
        }
        else
        {
            unsigned int numberOfLightSources;
            Build_Bounding_Slabs(&(sd->boundingSlabs), sd->objects, sd->numberOfFiniteObjects,
                                 sd->numberOfInfiniteObjects, numberOfLightSources);
        }
        for (ObjectPtr o : sd->objects)
            if (!(o->Type & LIGHT_SOURCE_OBJECT))
                NumberObjects(o, ids, flat);
    }

    void Hit(const Intersection& isect, int& obj, int& tri) const
    {
        obj = -1;
        tri = -1;
        auto it = ids.find(isect.Object);
        if (it != ids.end())
            obj = it->second;
        const Mesh *m = dynamic_cast<const Mesh *>(isect.Object);
        if (m != nullptr && isect.Pointer != nullptr)
            tri = (int)(reinterpret_cast<const MESH_TRIANGLE *>(isect.Pointer) - m->Data->Triangles);
    }
};

void PrintStats(TraceThreadData& td)
{
    RenderStatistics& st = td.Stats();
    std::printf("{\"number_of_rays\": %llu, \"shadow_ray_tests\": %llu, \"shadow_rays_succeeded\": %llu, "
                "\"reflected_rays\": %llu, \"shadow_cache_hits\": %llu, \"transmitted_rays\": %llu, "
                "\"media_samples\": %llu, \"media_intervals\": %llu, \"refracted_rays\": %llu, "
                "\"internal_reflected_rays\": %llu}\n",
                (unsigned long long)st[Number_Of_Rays], (unsigned long long)st[Shadow_Ray_Tests],
                (unsigned long long)st[Shadow_Rays_Succeeded], (unsigned long long)st[Reflected_Rays_Traced],
                (unsigned long long)st[Shadow_Cache_Hits], (unsigned long long)st[Transmitted_Rays_Traced],
                (unsigned long long)st[Media_Samples], (unsigned long long)st[Media_Intervals],
                (unsigned long long)st[Refracted_Rays_Traced], (unsigned long long)st[Internal_Reflected_Rays_Traced]);
}

void Vec(FILE *f, const char *name, const Vector3d& v)
{
    std::fprintf(f, "%s %.17g %.17g %.17g\n", name, v[X], v[Y], v[Z]);
}

} // namespace

static void OnSegv(int)
{
    void *frames[64];
    int n = backtrace(frames, 64);
    backtrace_symbols_fd(frames, n, 2);
    _exit(139);
}

int main(int argc, char **argv)
{
    if (std::getenv("POV_ORACLE_DEBUG"))
        std::signal(SIGSEGV, OnSegv);
    if (argc < 6)
    {
        std::fprintf(stderr, "usage: pov_oracle SCENE W H pixels|rays|scene|jitter ...\n");
        return 2;
    }
    const char *scene = argv[1];
    int width = std::atoi(argv[2]);
    int height = std::atoi(argv[3]);
    std::string mode = argv[4];

    if (mode == "jitter")
    {
        // the pretrace jitter table of RadiosityTask::Run (radiositytask.cpp:99):
        // RandomDoubleSequence(-1, 1, 2047), as the reference generates it
        pov::RandomDoubleSequence rands(-1.0, 1.0, 2047);
        FILE *f = std::fopen(argv[5], "wb");
        for (size_t i = 0; i < 2047; i++)
        {
            double v = rands(i);
            std::fwrite(&v, sizeof(v), 1, f);
        }
        std::fclose(f);
        return 0;
    }

    // the process-wide tables the renderer sets up at start-up
    // (povray_init, source/backend/povray.cpp:653-654): noise lattice and
    // permutations, pattern generators
    pov::Initialize_Noise();
    pov::InitializePatternGenerators();
    DefaultPlatformBase platform;  // file access for the parser (vfe provides this in the CLI)
    try
    {
        Harness h;
        h.Parse(scene, width, height);
        Trace::CooperateFunctor cooperate;
        Trace::RadiosityFunctor radiosity;
        QualityFlags quality(9);
        TraceThreadData td(h.sd, 0);
        // the pixel tracer with the renderer's own MediaFunction wired to it,
        // as TraceTask holds them (tracetask.h:122-126, tracetask.cpp:253)
        struct PixelTracer
        {
            TracePixel trace;
            MediaFunction media;
            PixelTracer(std::shared_ptr<SceneData> sd, TraceThreadData *td, const QualityFlags& q,
                        Trace::CooperateFunctor& coop, Trace::RadiosityFunctor& rad) :
                trace(sd, &sd->parsedCamera, td, sd->parsedMaxTraceLevel, sd->parsedAdcBailout, q, coop, media, rad),
                media(td, &trace, nullptr)
            {}
        } pt(h.sd, &td, quality, cooperate, radiosity);
        TracePixel& trace = pt.trace;

        if (mode == "pixels" || mode == "pixelstats")
        {
            // pixelstats: per pixel, the counters it added (rays, shadow
            // tests, shadow successes, media samples, media intervals)
            const bool per_pixel = (mode == "pixelstats");
            std::vector<uint64_t> counts;
            const int which[5] = {Number_Of_Rays, Shadow_Ray_Tests, Shadow_Rays_Succeeded, Media_Samples,
                                  Media_Intervals};
            std::vector<float> out((size_t)width * height * 4);
            for (int y = 0; y < height; y++)
                for (int x = 0; x < width; x++)
                {
                    RGBTColour col;
                    uint64_t before[5];
                    for (int k = 0; k < 5; k++)
                        before[k] = td.Stats()[(IntStatsIndex)which[k]];
                    trace(x + 0.5, y + 0.5, width, height, col);
                    if (per_pixel)
                        for (int k = 0; k < 5; k++)
                            counts.push_back(td.Stats()[(IntStatsIndex)which[k]] - before[k]);
                    float *p = &out[((size_t)y * width + x) * 4];
                    p[0] = col.red();
                    p[1] = col.green();
                    p[2] = col.blue();
                    p[3] = col.transm();
                }
            FILE *f = std::fopen(argv[5], "wb");
            if (per_pixel)
                std::fwrite(counts.data(), sizeof(uint64_t), counts.size(), f);
            else
                std::fwrite(out.data(), sizeof(float), out.size(), f);
            std::fclose(f);
            PrintStats(td);
        }
        else if (mode == "rays")
        {
            if (argc < 7)
                return 2;
            FILE *f = std::fopen(argv[5], "rb");
            int32_t n = 0;
            if (std::fread(&n, 4, 1, f) != 1)
                return 3;
            std::vector<double> rays((size_t)n * 6);
            if (std::fread(rays.data(), 8, rays.size(), f) != rays.size())
                return 3;
            std::fclose(f);
            FILE *o = std::fopen(argv[6], "wb");
            for (int32_t i = 0; i < n; i++)
            {
                const double *r = &rays[(size_t)i * 6];
                TraceTicket ticket(h.sd->parsedMaxTraceLevel, h.sd->parsedAdcBailout);
                Ray ray(ticket, Vector3d(r[0], r[1], r[2]), Vector3d(r[3], r[4], r[5]));
                Intersection isect;
                int32_t obj = -1, tri = -1;
                double depth = 0.0;
                if (trace.FindIntersection(isect, ray))
                {
                    h.Hit(isect, obj, tri);
                    depth = isect.Depth;
                }
                std::fwrite(&obj, 4, 1, o);
                std::fwrite(&tri, 4, 1, o);
                std::fwrite(&depth, 8, 1, o);
            }
            std::fclose(o);
            PrintStats(td);
        }
        else if (mode == "desc")
        {
            povgpu_ref::FlatScene flat;
            std::string why;
            if (!povgpu_ref::FlattenScene(*h.sd, flat, why))
            {
                std::fprintf(stderr, "pov_oracle: not flattened: %s\n", why.c_str());
                return 4;
            }
            if (!povgpu_ref::WriteSceneFile(flat, argv[5]))
                return 3;
            PrintStats(td);
        }
        else if (mode == "scene")
        {
            FILE *f = std::fopen(argv[5], "w");
            const Camera& cam = h.sd->parsedCamera;
            Vec(f, "location", cam.Location);
            Vec(f, "direction", cam.Direction);
            Vec(f, "right", cam.Right);
            Vec(f, "up", cam.Up);
            std::fprintf(f, "max_trace_level %u\nadc_bailout %.17g\n", h.sd->parsedMaxTraceLevel,
                         h.sd->parsedAdcBailout);
            std::fprintf(f, "objects %zu\n", h.flat.size());
            for (size_t i = 0; i < h.flat.size(); i++)
            {
                ObjectPtr o = h.flat[i];
                std::fprintf(f, "object %zu flags %u bbox %.9g %.9g %.9g %.9g %.9g %.9g\n", i,
                             (unsigned)o->Flags, o->BBox.lowerLeft[X], o->BBox.lowerLeft[Y],
                             o->BBox.lowerLeft[Z], o->BBox.size[X], o->BBox.size[Y], o->BBox.size[Z]);
            }
            std::fclose(f);
            PrintStats(td);
        }
        else
        {
            std::fprintf(stderr, "unknown mode %s\n", mode.c_str());
            return 2;
        }
    }
    catch (std::exception& e)
    {
        std::fprintf(stderr, "pov_oracle: %s\n", e.what());
        return 1;
    }
    return 0;
}
