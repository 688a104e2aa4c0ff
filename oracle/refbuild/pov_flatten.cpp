// pov_flatten.cpp -- SceneData -> PovGpuSceneDesc, compiled against the
// reference's headers (see pov_flatten.h).  Every field is read from the
// object the parser built; the comments name the reference member each ABI
// field carries.
#include "pov_flatten.h"

#include <algorithm>
#include <cstring>
#include <map>

#include "core/lighting/lightsource.h"
#include "core/lighting/radiosity.h"
#include "core/material/interior.h"
#include "core/material/media.h"
#include "core/material/normal.h"
#include "core/material/pattern.h"
#include "core/material/pigment.h"
#include "core/material/texture.h"
#include "core/material/warp.h"
#include "core/math/matrix.h"
#include "core/scene/camera.h"
#include "core/scene/object.h"
#include "core/scene/scenedata.h"
#include "core/shape/box.h"
#include "core/shape/csg.h"
#include "core/shape/mesh.h"
#include "core/shape/plane.h"
#include "core/shape/sphere.h"
#include "core/shape/torus.h"

using namespace pov;

namespace povgpu_ref {

namespace {

void Copy3(double* d, const Vector3d& v)
{
    d[0] = v[X];
    d[1] = v[Y];
    d[2] = v[Z];
}

void CopyMatrix(double* d, const MATRIX m)
{
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++)
            d[4 * i + j] = m[i][j];
}

struct Walker
{
    const SceneData& sd;
    FlatScene& out;
    std::string& why;
    std::map<const TEXTURE*, int> material_of;
    std::map<const Mesh_Data_Struct*, int> mesh_of;
    std::map<const Interior*, int> media_of;
    std::map<const Interior*, int> interior_of;

    // Interior (source/core/coretypes.h:193-215) after Interior::PostProcess;
    // one entry per distinct Interior object (CSG children share their
    // parent's), 1-based.
    int InteriorOf(const Interior* in)
    {
        if (in == nullptr)
            return 0;
        auto it = interior_of.find(in);
        if (it != interior_of.end())
            return it->second;
        PovGpuInterior d;
        std::memset(&d, 0, sizeof(d));
        d.ior = in->IOR;
        d.dispersion = in->Dispersion;
        d.caustics = in->Caustics;
        d.fade_distance = in->Fade_Distance;
        d.fade_power = in->Fade_Power;
        d.fade_colour[0] = in->Fade_Colour.Red();
        d.fade_colour[1] = in->Fade_Colour.Green();
        d.fade_colour[2] = in->Fade_Colour.Blue();
        d.old_refract = in->Old_Refract;
        out.interiors.push_back(d);
        const int idx = (int)out.interiors.size();
        interior_of[in] = idx;
        return idx;
    }

    bool Fail(int index, const std::string& what)
    {
        why = "object " + std::to_string(index) + ": " + what;
        return false;
    }

    // The ABI's pattern kind of a pattern object (the kinds the GPU path
    // takes), 0 for any other.  `normal`: the pattern stands in a normal,
    // where bumps is its own kind (in a pigment it is bozo's noise).
    static int PatternKind(const BasicPattern* p, bool normal)
    {
        if (dynamic_cast<const CheckerPattern*>(p)) return POV_PATTERN_CHECKER;
        if (dynamic_cast<const GradientPattern*>(p)) return POV_PATTERN_GRADIENT;
        if (dynamic_cast<const BumpsPattern*>(p)) return normal ? POV_PATTERN_BUMPS : POV_PATTERN_BOZO;
        if (dynamic_cast<const BozoPattern*>(p) || dynamic_cast<const SpottedPattern*>(p)) return POV_PATTERN_BOZO;
        if (dynamic_cast<const GranitePattern*>(p)) return POV_PATTERN_GRANITE;
        if (dynamic_cast<const MarblePattern*>(p)) return POV_PATTERN_MARBLE;
        if (dynamic_cast<const WoodPattern*>(p)) return POV_PATTERN_WOOD;
        if (dynamic_cast<const AgatePattern*>(p)) return POV_PATTERN_AGATE;
        if (dynamic_cast<const OnionPattern*>(p)) return POV_PATTERN_ONION;
        if (dynamic_cast<const LeopardPattern*>(p)) return POV_PATTERN_LEOPARD;
        if (dynamic_cast<const DentsPattern*>(p)) return POV_PATTERN_DENTS;
        if (dynamic_cast<const WrinklesPattern*>(p)) return POV_PATTERN_WRINKLES;
        if (dynamic_cast<const RipplesPattern*>(p)) return POV_PATTERN_RIPPLES;
        if (dynamic_cast<const WavesPattern*>(p)) return POV_PATTERN_WAVES;
        if (dynamic_cast<const RadialPattern*>(p)) return POV_PATTERN_RADIAL;
        if (dynamic_cast<const PlanarPattern*>(p)) return POV_PATTERN_PLANAR;
        if (dynamic_cast<const SphericalPattern*>(p)) return POV_PATTERN_SPHERICAL;
        if (dynamic_cast<const CylindricalPattern*>(p)) return POV_PATTERN_CYLINDRICAL;
        if (dynamic_cast<const BoxedPattern*>(p)) return POV_PATTERN_BOXED;
        if (dynamic_cast<const SquarePattern*>(p)) return POV_PATTERN_SQUARE;
        if (dynamic_cast<const TriangularPattern*>(p)) return POV_PATTERN_TRIANGULAR;
        if (dynamic_cast<const CubicPattern*>(p)) return POV_PATTERN_CUBIC;
        if (dynamic_cast<const HexagonPattern*>(p)) return POV_PATTERN_HEXAGON;
        if (dynamic_cast<const BrickPattern*>(p)) return POV_PATTERN_BRICK;
        if (dynamic_cast<const Spiral1Pattern*>(p)) return POV_PATTERN_SPIRAL1;
        if (dynamic_cast<const Spiral2Pattern*>(p)) return POV_PATTERN_SPIRAL2;
        if (dynamic_cast<const CellsPattern*>(p)) return POV_PATTERN_CELLS;
        if (dynamic_cast<const CracklePattern*>(p)) return POV_PATTERN_CRACKLE;
        if (dynamic_cast<const QuiltedPattern*>(p)) return POV_PATTERN_QUILTED;
        return 0;
    }

    // A pattern (BasicPattern, source/core/material/pattern.h:151-283, with
    // ContinuousPattern's wave and the kinds' own fields) and its warps as
    // the ABI takes them: the list the parser builds for `turbulence` and
    // transforms -- a ClassicTurbulence first, then one TransformWarp
    // (Warp_EPoint walks the list backwards: the transform, then the
    // turbulence).  `map`: the colour map (nullptr for a normal's pattern).
    // `fwd` receives the transform's forward matrix (identity without one).
    bool Pattern(const BasicPattern* p, bool normal, const ColourBlendMap* map, int index, PovGpuPattern& d,
                 double* fwd)
    {
        std::memset(&d, 0, sizeof(d));
        d.type = PatternKind(p, normal);
        if (d.type == 0)
            return Fail(index, "pattern kind the GPU path lacks");
        d.noise_generator = p->noiseGenerator != 0 ? p->noiseGenerator : sd.noiseGenerator;
        d.frequency = 1.0;
        d.phase = 0.0;
        d.exponent = 1.0;
        d.omega = 0.5;
        d.lambda = 2.0;
        d.octaves = 6;
        d.agate_turb = 1.0;
        if (const ContinuousPattern* c = dynamic_cast<const ContinuousPattern*>(p)) {
            if (c->waveType == kWaveType_Raw)
                return Fail(index, "raw pattern wave");
            d.wave_type = (int32_t)c->waveType - (int32_t)kWaveType_Ramp;   // ramp, sine, ... poly as POV_WAVE_*
            d.frequency = c->waveFrequency;
            d.phase = c->wavePhase;
            d.exponent = c->waveExponent;
        }
        if (const GradientPattern* g = dynamic_cast<const GradientPattern*>(p))
            Copy3(d.gradient, g->gradient);
        if (const AgatePattern* a = dynamic_cast<const AgatePattern*>(p))
            d.agate_turb = a->agateTurbScale;
        if (const BrickPattern* b = dynamic_cast<const BrickPattern*>(p)) {
            Copy3(d.brick_size, b->brickSize);
            d.mortar = b->mortar;
        }
        if (const SpiralPattern* sp = dynamic_cast<const SpiralPattern*>(p))
            d.arms = sp->arms;
        if (const CracklePattern* c = dynamic_cast<const CracklePattern*>(p)) {
            if (c->repeat.x() || c->repeat.y() || c->repeat.z())
                return Fail(index, "crackle repeat");
            Copy3(d.crackle_form, c->crackleForm);
            d.crackle_metric = c->crackleMetric;
            d.crackle_offset = c->crackleOffset;
            d.crackle_solid = c->crackleIsSolid ? 1 : 0;
        }
        if (const QuiltedPattern* q = dynamic_cast<const QuiltedPattern*>(p)) {
            d.control0 = q->Control0;
            d.control1 = q->Control1;
        }
        MATRIX ident;
        MIdentity(ident);
        CopyMatrix(d.inverse, ident);
        CopyMatrix(fwd, ident);
        for (size_t k = 0; k < p->warps.size(); k++) {
            const GenericWarp* w = p->warps[k];
            if (const ClassicTurbulence* t = dynamic_cast<const ClassicTurbulence*>(w)) {
                if (k != 0)
                    return Fail(index, "turbulence after another warp");
                d.has_turbulence = 1;
                Copy3(d.turbulence, t->Turbulence);
                d.octaves = t->Octaves;
                d.omega = t->Omega;
                d.lambda = t->Lambda;
            } else if (const TransformWarp* tw = dynamic_cast<const TransformWarp*>(w)) {
                if (k + 1 != p->warps.size())
                    return Fail(index, "warp after the pattern's transform");
                CopyMatrix(d.inverse, tw->Trans.inverse);
                CopyMatrix(fwd, tw->Trans.matrix);
            } else {
                return Fail(index, "warp the GPU path lacks");
            }
        }
        if (map != nullptr) {
            const auto& e = map->Blend_Map_Entries;
            if (e.empty() || e.size() > POV_PATTERN_MAX_ENTRIES)
                return Fail(index, "colour map size");
            d.num_entries = (int32_t)e.size();
            for (size_t k = 0; k < e.size(); k++) {
                d.filters[k] = e[k].Vals.filter();
                d.transmits[k] = e[k].Vals.transm();
                d.values[k] = e[k].value;
                d.colours[k][0] = e[k].Vals.colour().Red();
                d.colours[k][1] = e[k].Vals.colour().Green();
                d.colours[k][2] = e[k].Vals.colour().Blue();
            }
        }
        return true;
    }

    // A texture's pigment pattern (Compute_Pigment's pattern path,
    // source/core/material/pigment.cpp:395-475): its colour map, or the
    // pattern's default one; 1-based index into the patterns.
    bool PigmentPattern(const PIGMENT* pig, int index, int& out_index)
    {
        const ColourBlendMap* map = nullptr;
        ColourBlendMapConstPtr def;
        if (pig->Blend_Map) {
            map = dynamic_cast<const ColourBlendMap*>(pig->Blend_Map.get());
            if (map == nullptr)
                return Fail(index, "pigment map (not a colour map)");
        } else {
            def = pig->pattern->GetDefaultBlendMap();
            map = def.get();
            if (map == nullptr)
                return Fail(index, "pattern without a colour map");
        }
        PovGpuPattern d;
        double fwd[16];
        if (!Pattern(pig->pattern.get(), false, map, index, d, fwd))
            return false;
        out.patterns.push_back(d);
        out_index = (int)out.patterns.size();
        return true;
    }

    // A texture's normal (Tnormal_Struct, normal.h:118-123, perturbed by
    // Perturb_Normal, normal.cpp:784-905): its pattern, Amount, Delta, the
    // no_bump_scale flag and the pattern transform's forward matrix;
    // 1-based index into the normals.
    bool NormalOf(const TNORMAL* n, int index, int& out_index)
    {
        if (n->Blend_Map)
            return Fail(index, "normal map or slope map");
        const bool special = n->Type == BUMPS_PATTERN || n->Type == DENTS_PATTERN || n->Type == WRINKLES_PATTERN ||
                             n->Type == RIPPLES_PATTERN || n->Type == WAVES_PATTERN;
        if (!special && n->Type != GENERIC_PATTERN)
            return Fail(index, "normal pattern kind the GPU path lacks");
        PovGpuPattern p;
        PovGpuNormal d;
        std::memset(&d, 0, sizeof(d));
        if (!Pattern(n->pattern.get(), true, nullptr, index, p, d.matrix))
            return false;
        out.patterns.push_back(p);
        d.pattern = (int32_t)out.patterns.size();
        d.dont_scale_bumps = (n->Flags & DONT_SCALE_BUMPS_FLAG) ? 1 : 0;
        d.amount = n->Amount;
        d.delta = n->Delta;
        out.normals.push_back(d);
        out_index = (int)out.normals.size();
        return true;
    }

    // TEXTURE + its FINISH (source/core/material/texture.h:108-141) as the
    // ABI's single-layer material: a plain pigment colour and the finish
    // values as the parser leaves them.
    bool Material(const TEXTURE* t, int index, int& mat)
    {
        auto it = material_of.find(t);
        if (it != material_of.end())
        {
            mat = it->second;
            return true;
        }
        if (t == nullptr || t->Type != PLAIN_PATTERN || t->Next != nullptr)
            return Fail(index, "layered or mapped texture");
        if (t->Pigment == nullptr || (t->Pigment->Type != PLAIN_PATTERN && !t->Pigment->pattern))
            return Fail(index, "pigment without a pattern");
        int pattern = 0, normal = 0;
        if (t->Pigment->Type != PLAIN_PATTERN && !PigmentPattern(t->Pigment, index, pattern))
            return false;
        if (t->Tnormal != nullptr && !NormalOf(t->Tnormal, index, normal))
            return false;
        const FINISH* f = t->Finish;
        PovGpuMaterial m;
        std::memset(&m, 0, sizeof(m));
        const TransColour& c = t->Pigment->colour;
        m.pigment[0] = c.colour().Red();
        m.pigment[1] = c.colour().Green();
        m.pigment[2] = c.colour().Blue();
        m.pigment[3] = c.filter();
        m.pigment[4] = c.transm();
        m.ambient[0] = f->Ambient.Red();
        m.ambient[1] = f->Ambient.Green();
        m.ambient[2] = f->Ambient.Blue();
        m.emission[0] = f->Emission.Red();
        m.emission[1] = f->Emission.Green();
        m.emission[2] = f->Emission.Blue();
        m.diffuse = f->Diffuse;
        m.diffuse_back = f->DiffuseBack;
        m.brilliance = f->Brilliance;
        m.brilliance_adjust = f->BrillianceAdjust;
        m.brilliance_adjust_rad = f->BrillianceAdjustRad;
        m.phong = f->Phong;
        m.phong_size = f->Phong_Size;
        m.specular = f->Specular;
        m.roughness = f->Roughness;            // stored inverted by the parser
        m.metallic = f->Metallic;
        m.reflection_max[0] = f->Reflection_Max.Red();
        m.reflection_max[1] = f->Reflection_Max.Green();
        m.reflection_max[2] = f->Reflection_Max.Blue();
        m.reflection_min[0] = f->Reflection_Min.Red();
        m.reflection_min[1] = f->Reflection_Min.Green();
        m.reflection_min[2] = f->Reflection_Min.Blue();
        m.reflection_falloff = f->Reflection_Falloff;
        m.reflect_exp = f->Reflect_Exp;
        m.reflect_metallic = f->Reflect_Metallic;
        m.reflection_fresnel = f->Reflection_Fresnel ? 1 : 0;
        m.conserve_energy = f->Conserve_Energy;
        m.fresnel = f->Fresnel;
        m.crand = f->Crand;
        m.irid = f->Irid;
        m.pattern = pattern;
        m.normal = normal;
        mat = (int)out.materials.size();
        out.materials.push_back(m);
        material_of[t] = mat;
        return true;
    }

    // Mesh_Data_Struct (source/core/shape/mesh.h:107-119) of a mesh2 back in
    // the form its SDL gave it: the vertex_vectors; the normal_vectors
    // without the per-triangle face normals Parse_Mesh2 appends after them
    // (source/parser/parser.cpp:4568-4575); face and normal index triples in
    // their parsed order -- Compute_Mesh_Triangle (mesh.cpp:838-982) may
    // have exchanged P1/P2 (and N1/N2), which shows as the stored order's
    // normal pointing against the triangle's recorded face normal, and is
    // undone here so that the library's own Compute_Mesh_Triangle sees what
    // the parser saw.
    int MeshData(const Mesh* m)
    {
        auto it = mesh_of.find(m->Data);
        if (it != mesh_of.end())
            return it->second;
        const Mesh_Data_Struct* d = m->Data;
        const int nv = d->Number_Of_Vertices, nt = d->Number_Of_Triangles;
        const int nn = d->Number_Of_Normals > nt ? d->Number_Of_Normals - nt : 0;
        std::vector<float> v((size_t)nv * 3), n((size_t)nn * 3);
        for (int i = 0; i < nv; i++)
            for (int k = 0; k < 3; k++)
                v[3 * (size_t)i + k] = d->Vertices[i][k];
        for (int i = 0; i < nn; i++)
            for (int k = 0; k < 3; k++)
                n[3 * (size_t)i + k] = d->Normals[i][k];
        std::vector<int32_t> f((size_t)nt * 3), fn((size_t)nt * 3);
        for (int i = 0; i < nt; i++)
        {
            const MESH_TRIANGLE& t = d->Triangles[i];
            int32_t p1 = t.P1, p2 = t.P2, p3 = t.P3, n1 = t.N1, n2 = t.N2, n3 = t.N3;
            const Vector3d P1(d->Vertices[p1]), P2(d->Vertices[p2]), P3(d->Vertices[p3]);
            const Vector3d N = cross(P3 - P1, P2 - P1);   // the face normal's direction for this order
            if (dot(N, Vector3d(d->Normals[t.Normal_Ind])) < 0.0)
            {
                std::swap(p1, p2);
                if (t.Smooth)
                    std::swap(n1, n2);
            }
            f[3 * (size_t)i] = p1;
            f[3 * (size_t)i + 1] = p2;
            f[3 * (size_t)i + 2] = p3;
            fn[3 * (size_t)i] = n1;
            fn[3 * (size_t)i + 1] = n2;
            fn[3 * (size_t)i + 2] = n3;
        }
        const int idx = (int)out.meshes.size();
        out.mesh_vertices.push_back(std::move(v));
        out.mesh_normals.push_back(std::move(n));
        out.mesh_faces.push_back(std::move(f));
        out.mesh_normal_indices.push_back(std::move(fn));
        PovGpuMesh pm;
        std::memset(&pm, 0, sizeof(pm));
        pm.num_vertices = nv;
        pm.num_normals = nn;
        pm.num_triangles = nt;
        out.meshes.push_back(pm);
        mesh_of[m->Data] = idx;
        return idx;
    }

    // Interior media (source/core/coretypes.h:141-182, after
    // Media::PostProcess): constant isotropic media only.
    bool MediaOf(const Interior* in, int index, int& media)
    {
        media = 0;
        if (in == nullptr || in->media.empty())
            return true;
        auto it = media_of.find(in);
        if (it != media_of.end())
        {
            media = it->second;
            return true;
        }
        if (in->media.size() != 1)
            return Fail(index, "more than one media");
        const Media& md = in->media[0];
        if (!md.Density.empty())
            return Fail(index, "media density pattern");
        PovGpuMedia m;
        std::memset(&m, 0, sizeof(m));
        m.scattering_type = md.Type;
        m.method = (int32_t)md.Sample_Method;
        m.intervals = md.Intervals;
        m.min_samples = md.Min_Samples;
        m.max_samples = md.Max_Samples;
        m.aa_level = md.AA_Level;
        m.aa_threshold = (float)md.AA_Threshold;
        m.jitter = (float)md.Jitter;
        const MathColour* src[4] = {&md.Absorption, &md.Emission, &md.Scattering, &md.Extinction};
        float* dst[4] = {m.absorption, m.emission, m.scattering, m.extinction};
        for (int k = 0; k < 4; k++)
        {
            dst[k][0] = src[k]->Red();
            dst[k][1] = src[k]->Green();
            dst[k][2] = src[k]->Blue();
        }
        m.eccentricity = (float)md.Eccentricity;
        out.medias.push_back(m);
        media = (int)out.medias.size();   // 1-based in PovGpuObject
        media_of[in] = media;
        return true;
    }

    bool Object(ObjectPtr o, int parent)
    {
        const int index = (int)out.objects.size();
        out.objects.emplace_back();
        out.object_interior.push_back(InteriorOf(o->interior.get()));
        PovGpuObject d;
        std::memset(&d, 0, sizeof(d));
        d.parent = parent;
        d.first_child = -1;
        d.mesh = -1;
        d.flags = (Test_Flag(o, INVERTED_FLAG) ? POV_FLAG_INVERTED : 0) |
                  (Test_Flag(o, NO_SHADOW_FLAG) ? POV_FLAG_NO_SHADOW : 0) |
                  (Test_Flag(o, INFINITE_FLAG) ? POV_FLAG_INFINITE : 0) |
                  (Test_Flag(o, DOUBLE_ILLUMINATE_FLAG) ? POV_FLAG_DOUBLE_ILLUM : 0) |
                  (Test_Flag(o, NO_REFLECTION_FLAG) ? POV_FLAG_NO_REFLECTION : 0) |
                  (Test_Flag(o, NO_IMAGE_FLAG) ? POV_FLAG_NO_IMAGE : 0) |
                  (Test_Flag(o, HOLLOW_FLAG) ? POV_FLAG_HOLLOW : 0);
        if (o->Trans != nullptr)
        {
            d.flags |= POV_FLAG_HAS_TRANS;
            CopyMatrix(d.trans, o->Trans->matrix);
            CopyMatrix(d.trans + 16, o->Trans->inverse);
        }
        if (!o->Clip.empty() || !o->Bound.empty())
            return Fail(index, "clipped_by / bounded_by");
        d.material = -1;
        const CSG* csg = dynamic_cast<const CSG*>(o);
        if (o->Texture != nullptr && !Material(o->Texture, index, d.material))
            return false;
        if (!MediaOf(o->interior.get(), index, d.media))
            return false;
        if (const Sphere* s = dynamic_cast<const Sphere*>(o))
        {
            d.type = POV_OBJ_SPHERE;     // Sphere::Center, Radius
            Copy3(d.p, s->Center);
            d.p[3] = s->Radius;
        }
        else if (const Plane* p = dynamic_cast<const Plane*>(o))
        {
            d.type = POV_OBJ_PLANE;      // Plane::Normal_Vector, Distance
            Copy3(d.p, p->Normal_Vector);
            d.p[3] = p->Distance;
        }
        else if (const Box* b = dynamic_cast<const Box*>(o))
        {
            d.type = POV_OBJ_BOX;        // Box::bounds
            Copy3(d.p, b->bounds[0]);
            Copy3(d.p + 3, b->bounds[1]);
        }
        else if (const Torus* t = dynamic_cast<const Torus*>(o))
        {
            d.type = POV_OBJ_TORUS;      // Torus::MajorRadius, MinorRadius (+ Trans)
            d.p[0] = t->MajorRadius;
            d.p[1] = t->MinorRadius;
        }
        else if (const Mesh* m = dynamic_cast<const Mesh*>(o))
        {
            d.type = POV_OBJ_MESH;
            d.mesh = MeshData(m);
        }
        else if (dynamic_cast<const CSGMerge*>(o) != nullptr)   // before CSGUnion: it derives from it
            d.type = POV_OBJ_MERGE;
        else if (dynamic_cast<const CSGIntersection*>(o) != nullptr)   // intersection and difference
            d.type = POV_OBJ_INTERSECTION;
        else if (dynamic_cast<const CSGUnion*>(o) != nullptr)
            d.type = POV_OBJ_UNION;
        else
            return Fail(index, "object type the GPU path does not take");
        out.objects[index] = d;
        if (csg != nullptr)
        {
            out.objects[index].num_children = (int32_t)csg->children.size();
            for (ObjectPtr c : csg->children)
            {
                if (out.objects[index].first_child < 0)
                    out.objects[index].first_child = (int32_t)out.objects.size();
                if (!Object(c, index))
                    return false;
            }
        }
        return true;
    }
};

}  // namespace

bool FlattenScene(const SceneData& sd, FlatScene& out, std::string& why)
{
    out = FlatScene();
    Walker w{sd, out, why, {}, {}, {}};
    for (ObjectPtr o : sd.objects)
        if (!(o->Type & LIGHT_SOURCE_OBJECT))
            if (!w.Object(o, -1))
                return false;
    // light sources (LightSource, source/core/scene/object.h:313-351)
    for (const LightSource* l : sd.lightSources)
    {
        if (l->Projected_Through_Object != nullptr || l->Use_Full_Area_Lighting || l->Media_Attenuation ||
            (l->Light_Type != POINT_SOURCE && l->Light_Type != SPOT_SOURCE && l->Light_Type != FILL_LIGHT_SOURCE &&
             l->Light_Type != CYLINDER_SOURCE))
        {
            why = "light source of a kind the GPU path does not take";
            return false;
        }
        PovGpuLight g;
        std::memset(&g, 0, sizeof(g));
        Copy3(g.center, l->Center);
        g.colour[0] = l->colour.Red();
        g.colour[1] = l->colour.Green();
        g.colour[2] = l->colour.Blue();
        g.kind = l->Area_Light ? POV_LIGHT_AREA : POV_LIGHT_POINT;
        g.adaptive_level = l->Adaptive_Level;
        if (l->Area_Light)
        {
            Copy3(g.axis1, l->Axis1);
            Copy3(g.axis2, l->Axis2);
            g.area_size1 = l->Area_Size1;
            g.area_size2 = l->Area_Size2;
            g.jitter = l->Jitter ? 1 : 0;
            g.circular = l->Circular ? 1 : 0;
            g.orient = l->Orient ? 1 : 0;
        }
        g.fade_distance = l->Fade_Distance;
        g.fade_power = l->Fade_Power;
        // Light_Type numbers are the ABI's (lightsource.h:78-81)
        g.light_type = l->Light_Type;
        g.parallel = l->Parallel ? 1 : 0;
        Copy3(g.points_at, l->Points_At);
        g.radius = l->Radius;
        g.falloff = l->Falloff;
        g.tightness = l->Coeff;
        out.lights.push_back(g);
    }
    PovGpuSceneDesc& d = out.desc;
    std::memset(&d, 0, sizeof(d));
    d.abi_version = POV_GPU_ABI_VERSION;
    // the parsed camera (Camera, source/core/scene/camera.h)
    const Camera& cam = sd.parsedCamera;
    if (cam.Type != PERSPECTIVE_CAMERA)
    {
        why = "camera type";
        return false;
    }
    Copy3(d.camera.location, cam.Location);
    Copy3(d.camera.direction, cam.Direction);
    Copy3(d.camera.right, cam.Right);
    Copy3(d.camera.up, cam.Up);
    d.camera.type = 0;
    d.background[0] = sd.backgroundColour.colour().Red();
    d.background[1] = sd.backgroundColour.colour().Green();
    d.background[2] = sd.backgroundColour.colour().Blue();
    d.background[3] = sd.backgroundColour.transm();
    d.ambient_light[0] = sd.ambientLight.Red();
    d.ambient_light[1] = sd.ambientLight.Green();
    d.ambient_light[2] = sd.ambientLight.Blue();
    d.max_trace_level = (int32_t)sd.parsedMaxTraceLevel;
    d.adc_bailout = (float)sd.parsedAdcBailout;
    d.language_version = sd.languageVersion;
    // SceneRadiositySettings (source/core/lighting/radiosity.h:107-166)
    const SceneRadiositySettings& r = sd.radiositySettings;
    d.radiosity.enabled = r.radiosityEnabled ? 1 : 0;
    d.radiosity.count = (int32_t)r.count;
    d.radiosity.recursion_limit = r.recursionLimit;
    d.radiosity.nearest_count = (int32_t)r.nearestCount;
    d.radiosity.error_bound = r.errorBound;
    d.radiosity.low_error_factor = r.lowErrorFactor;
    d.radiosity.gray_threshold = r.grayThreshold;
    d.radiosity.minimum_reuse = r.minimumReuse;
    d.radiosity.maximum_reuse = r.maximumReuse;
    d.radiosity.brightness = r.brightness;
    d.radiosity.pretrace_start = r.pretraceStart;
    d.radiosity.pretrace_end = r.pretraceEnd;
    d.radiosity.adc_bailout = r.adcBailout;
    d.radiosity.always_sample = r.alwaysSample ? 1 : 0;
    d.radiosity.normal = r.normal ? 1 : 0;
    d.radiosity.media = r.media ? 1 : 0;
    for (size_t i = 0; i < out.meshes.size(); i++)
    {
        PovGpuMesh& m = out.meshes[i];
        m.vertices = out.mesh_vertices[i].data();
        m.normals = m.num_normals > 0 ? out.mesh_normals[i].data() : nullptr;
        m.face_indices = out.mesh_faces[i].data();
        m.normal_indices = m.num_normals > 0 ? out.mesh_normal_indices[i].data() : nullptr;
    }
    d.num_objects = (int32_t)out.objects.size();
    d.objects = out.objects.data();
    d.num_materials = (int32_t)out.materials.size();
    d.materials = out.materials.data();
    d.num_lights = (int32_t)out.lights.size();
    d.lights = out.lights.data();
    d.num_meshes = (int32_t)out.meshes.size();
    d.meshes = out.meshes.data();
    d.num_medias = (int32_t)out.medias.size();
    d.medias = out.medias.data();
    d.num_patterns = (int32_t)out.patterns.size();
    d.patterns = out.patterns.data();
    d.num_normals = (int32_t)out.normals.size();
    d.normals = out.normals.data();
    d.num_interiors = (int32_t)out.interiors.size();
    d.interiors = out.interiors.data();
    d.object_interior = out.object_interior.data();
    d.atmosphere_ior = sd.atmosphereIOR;
    return true;
}

namespace {

template <typename T> void Put(std::FILE* f, const T& v) { std::fwrite(&v, sizeof(T), 1, f); }

template <typename T> void PutArray(std::FILE* f, const std::vector<T>& v)
{
    Put(f, (uint32_t)v.size());
    if (!v.empty())
        std::fwrite(v.data(), sizeof(T), v.size(), f);
}

}  // namespace

bool WriteSceneFile(const FlatScene& fs, const char* path)
{
    std::FILE* f = std::fopen(path, "wb");
    if (f == nullptr)
        return false;
    const PovGpuSceneDesc& d = fs.desc;
    std::fwrite("PGSF", 1, 4, f);
    Put(f, (uint32_t)2);
    Put(f, (uint32_t)POV_GPU_ABI_VERSION);
    Put(f, d.camera);
    std::fwrite(d.background, sizeof(float), 4, f);
    std::fwrite(d.ambient_light, sizeof(float), 3, f);
    Put(f, d.max_trace_level);
    Put(f, d.adc_bailout);
    Put(f, d.language_version);
    Put(f, d.radiosity);
    PutArray(f, fs.objects);
    PutArray(f, fs.materials);
    PutArray(f, fs.lights);
    PutArray(f, fs.medias);
    PutArray(f, fs.patterns);
    PutArray(f, fs.normals);
    PutArray(f, fs.interiors);
    PutArray(f, fs.object_interior);
    Put(f, d.atmosphere_ior);
    Put(f, (uint32_t)fs.meshes.size());
    for (size_t i = 0; i < fs.meshes.size(); i++)
    {
        const PovGpuMesh& m = fs.meshes[i];
        const int32_t has_nidx = m.num_normals > 0 ? 1 : 0;
        Put(f, m.num_vertices);
        Put(f, m.num_normals);
        Put(f, m.num_triangles);
        Put(f, has_nidx);
        std::fwrite(fs.mesh_vertices[i].data(), sizeof(float), fs.mesh_vertices[i].size(), f);
        std::fwrite(fs.mesh_normals[i].data(), sizeof(float), fs.mesh_normals[i].size(), f);
        std::fwrite(fs.mesh_faces[i].data(), sizeof(int32_t), fs.mesh_faces[i].size(), f);
        if (has_nidx)
            std::fwrite(fs.mesh_normal_indices[i].data(), sizeof(int32_t), fs.mesh_normal_indices[i].size(), f);
    }
    const bool ok = std::ferror(f) == 0;
    std::fclose(f);
    return ok;
}

}  // namespace povgpu_ref
