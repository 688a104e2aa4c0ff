/*
 * povgpu.h -- C ABI of the GB300 trace path (libpovgpu.so).
 *
 * The reference renders a parsed scene by running one TraceTask per worker
 * thread; each task pulls 32x32 render blocks from the view
 * (ViewData::GetNextRectangle, source/backend/scene/view.cpp:236), traces
 * every pixel through TracePixel/Trace::TraceRay
 * (source/core/render/tracepixel.cpp:311, source/core/render/trace.cpp:135)
 * and hands the finished block back (ViewData::CompletedRectangle,
 * source/backend/scene/view.cpp:405).  This library replaces the per-pixel
 * part of that loop: the host walks SceneData once, fills a PovGpuSceneDesc,
 * and then submits whole batches of blocks.  Everything below the block
 * boundary (bounding-tree traversal, the All_Intersections/Inside tests,
 * shadow rays, Phong/specular shading, reflection, adaptive antialiasing,
 * radiosity) runs in CUDA kernels for sm_103a.
 *
 * Conventions:
 *   - every entry point returns int: 0 on success, a negative POV_GPU_E_*
 *     code on failure.  No C++ exception crosses this boundary.
 *   - all arrays are caller-owned and only read during the call unless the
 *     entry point says otherwise; device memory is owned by the library.
 *   - a scene handle may be used from several host threads; calls on one
 *     handle are serialised by an internal mutex.
 */
#ifndef POVGPU_H
#define POVGPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define POV_GPU_ABI_VERSION 3

/* ---- status codes ------------------------------------------------------- */
#define POV_GPU_OK              0
#define POV_GPU_E_INVALID      -1  /* bad argument or malformed description    */
#define POV_GPU_E_UNSUPPORTED  -2  /* object/material/light the GPU path lacks */
#define POV_GPU_E_CUDA         -3  /* a CUDA runtime call failed               */
#define POV_GPU_E_TIMEOUT      -4  /* host wait exceeded its limit             */
#define POV_GPU_E_NOMEM        -5  /* device allocation failed                 */
#define POV_GPU_E_DEVICE       -6  /* a kernel raised its device error word    */
#define POV_GPU_E_NODEVICE     -7  /* no CUDA device visible                   */
#define POV_GPU_E_CAPACITY     -8  /* request above a fixed scratch capacity;
                                      also a frame whose rays cross more than
                                      64 surfaces straight on at one trace
                                      level (transparent scenes)           */

/* ---- object types (subset of the reference's ObjectBase zoo) ------------ */
#define POV_OBJ_SPHERE        1   /* source/core/shape/sphere.cpp   */
#define POV_OBJ_PLANE         2   /* source/core/shape/plane.cpp    */
#define POV_OBJ_BOX           3   /* source/core/shape/box.cpp      */
#define POV_OBJ_MESH          4   /* source/core/shape/mesh.cpp     */
#define POV_OBJ_TORUS         5   /* source/core/shape/torus.cpp    */
#define POV_OBJ_UNION         6   /* CSGUnion, source/core/shape/csg.cpp        */
#define POV_OBJ_INTERSECTION  7   /* CSGIntersection (difference = intersection
                                     with children 2..n inverted, as the parser
                                     builds it: source/parser/parser.cpp:2224) */
#define POV_OBJ_MERGE         8   /* CSGMerge                                  */

/* ---- object flags (meaning of the reference's object.h:88-117 bits) ----- */
#define POV_FLAG_INVERTED       0x0001  /* INVERTED_FLAG                      */
#define POV_FLAG_NO_SHADOW      0x0002  /* NO_SHADOW_FLAG                     */
#define POV_FLAG_HAS_TRANS      0x0004  /* object carries a TRANSFORM         */
#define POV_FLAG_INFINITE       0x0008  /* INFINITE_FLAG (unbounded object)   */
#define POV_FLAG_DOUBLE_ILLUM   0x0010  /* DOUBLE_ILLUMINATE_FLAG             */
#define POV_FLAG_NO_REFLECTION  0x0020  /* NO_REFLECTION_FLAG                 */
#define POV_FLAG_NO_IMAGE       0x0040  /* NO_IMAGE_FLAG                      */
#define POV_FLAG_HOLLOW         0x0080  /* HOLLOW_FLAG (Interior::hollow)     */

/*
 * One object of SceneData::objects, flattened in depth-first order: a CSG
 * node is followed immediately by its children (recursively), so the hit
 * object id reported by the library is the index in this array of the leaf
 * primitive that was hit (Intersection::Object in the reference).
 *
 * Parameter layout of p[] by type:
 *   SPHERE  p[0..2] centre, p[3] radius
 *   PLANE   p[0..2] normal, p[3] Distance (the reference's stored value, i.e.
 *           minus the SDL offset: plane{y,-10} stores Distance=+10)
 *   BOX     p[0..2] corner1 (min), p[3..5] corner2 (max)
 *   TORUS   p[0] major radius, p[1] minor radius (always with a transform)
 *   MESH    mesh = index into PovGpuSceneDesc.meshes
 *   CSG     first_child/num_children index this array
 * media is the object's interior media: 1 + index into
 * PovGpuSceneDesc.medias, 0 = none.
 * trans[] is the object's TRANSFORM as two row-major 4x4 matrices:
 * trans[0..15] = forward matrix (object -> world), trans[16..31] = inverse.
 */
typedef struct PovGpuObject {
    int32_t type;
    int32_t flags;
    int32_t material;      /* index into materials; -1 = inherit from parent */
    int32_t parent;        /* index of the enclosing CSG object, -1 at top    */
    int32_t first_child;
    int32_t num_children;
    int32_t mesh;
    int32_t media;         /* 1 + index into medias, 0 = no interior media */
    double  p[8];
    double  trans[32];
} PovGpuObject;

/*
 * Texture of an object: a plain rgb pigment and a finish (the subset of
 * FINISH, source/core/material/texture.h, that the GPU path shades).  Values
 * are stored as the parser leaves them, e.g. roughness is 1/roughness.
 */
typedef struct PovGpuMaterial {
    float pigment[5];          /* r g b filter transmit                       */
    float ambient[3];
    float emission[3];
    float diffuse;
    float diffuse_back;
    float brilliance;
    float brilliance_adjust;   /* FINISH::BrillianceAdjust                    */
    float brilliance_adjust_rad;
    float phong;
    float phong_size;
    float specular;
    float roughness;           /* stored inverted, as the parser does         */
    float metallic;
    float reflection_max[3];
    float reflection_min[3];
    float reflection_falloff;
    float reflect_exp;
    float reflect_metallic;
    int32_t reflection_fresnel;
    int32_t conserve_energy;
    float fresnel;
    float crand;
    float irid;
    int32_t pattern;           /* pigment pattern: 1-based index into the scene's
                                  patterns, 0 = the plain pigment above       */
    int32_t normal;            /* normal perturbation: 1-based index into the
                                  scene's normals, 0 = the surface's own      */
} PovGpuMaterial;

/* Pattern pigments (PIGMENT with a pattern and a colour map: Compute_Pigment,
 * source/core/material/pigment.cpp:395-475; patterns in
 * source/core/material/pattern.cpp, noise and turbulence in noise.cpp /
 * portablenoise.cpp).  The point goes through the pattern's warps as
 * Warp_EPoint applies them (warp.cpp:103-122): the inverse TRANSFORM, then
 * the classic turbulence (GenericTurbulenceWarp::WarpPoint, warp.cpp:553-558,
 * which the parser keeps first in the list); continuous patterns take their
 * wave (ContinuousPattern::Evaluate, pattern.cpp:354-390); the colour map
 * blends linearly between its entries (BlendMap::Search,
 * pattern.cpp:1068-1109).  Opaque colours only. */
#define POV_PATTERN_CHECKER   1   /* CheckerPattern::Evaluate, pattern.cpp:5691      */
#define POV_PATTERN_GRADIENT  2   /* GradientPattern::EvaluateRaw, pattern.cpp:6386  */
#define POV_PATTERN_BOZO      3   /* bozo / spotted: NoisePattern, pattern.cpp:7858  */
#define POV_PATTERN_GRANITE   4   /* GranitePattern::EvaluateRaw, pattern.cpp:6429   */
#define POV_PATTERN_MARBLE    5   /* MarblePattern::EvaluateRaw, pattern.cpp:7831    */
#define POV_PATTERN_WOOD      6   /* WoodPattern::EvaluateRaw, pattern.cpp:8651      */
#define POV_PATTERN_AGATE     7   /* AgatePattern::EvaluateRaw, pattern.cpp:5396     */
#define POV_PATTERN_ONION     8   /* OnionPattern::EvaluateRaw, pattern.cpp:7934     */
#define POV_PATTERN_LEOPARD   9   /* LeopardPattern::EvaluateRaw, pattern.cpp:7179   */
/* normal-only patterns (the special normals of Perturb_Normal,
 * source/core/material/normal.cpp:855-878) */
#define POV_PATTERN_BUMPS    10   /* bumps, normal.cpp:235-246                       */
#define POV_PATTERN_DENTS    11   /* dents, normal.cpp:272-288                       */
#define POV_PATTERN_WRINKLES 12   /* wrinkles, normal.cpp:325-346                    */
/* pigment or normal: a continuous pattern as a pigment (RipplesPattern /
 * WavesPattern::EvaluateRaw, pattern.cpp:8163-8186 / 8593-8618), the special
 * normal of Perturb_Normal as a normal (ripples / waves, normal.cpp:130-225);
 * over the scene's 10 wave sources (number_of_waves 10, Initialize_Waves,
 * noise.cpp:189-205) */
#define POV_PATTERN_RIPPLES  13
#define POV_PATTERN_WAVES    14
/* geometric patterns (pattern.cpp; the last four through CLIP_DENSITY,
 * pattern.cpp:85); dents and wrinkles are pigments too (DentsPattern /
 * WrinklesPattern::EvaluateRaw, pattern.cpp:6307-6313 / 8720-8770) */
#define POV_PATTERN_RADIAL      15   /* RadialPattern::EvaluateRaw, pattern.cpp:8115   */
#define POV_PATTERN_PLANAR      16   /* PlanarPattern::EvaluateRaw, pattern.cpp:8024   */
#define POV_PATTERN_SPHERICAL   17   /* SphericalPattern::EvaluateRaw, pattern.cpp:8551 */
#define POV_PATTERN_CYLINDRICAL 18   /* CylindricalPattern::EvaluateRaw, pattern.cpp:6025 */
#define POV_PATTERN_BOXED       19   /* BoxedPattern::EvaluateRaw, pattern.cpp:5454    */
/* discrete patterns with a colour list (pigments only, like checker; no
 * wave): 4, 6 and 6 entries at the values 0..n-1 */
#define POV_PATTERN_SQUARE      20   /* SquarePattern::Evaluate, pattern.cpp:6740      */
#define POV_PATTERN_TRIANGULAR  21   /* TriangularPattern::Evaluate, pattern.cpp:6799  */
#define POV_PATTERN_CUBIC       22   /* CubicPattern::Evaluate, pattern.cpp:6699       */
#define POV_PATTERN_HEXAGON     23   /* HexagonPattern::Evaluate, pattern.cpp:6512 (3) */
/* brick: discrete, two entries (mortar, brick), brick_size and mortar;
 * spiral1 / spiral2: continuous with `arms` (triangle wave by default);
 * cells: continuous, each unit cube's value from the reference's pattern
 * random table (RandomDoubleSequence(0, 1, 32768): boost's mt19937 at its
 * default seed through uniform_real, randomsequence.cpp:138-149) */
#define POV_PATTERN_BRICK       24   /* BrickPattern::Evaluate, pattern.cpp:5495 (2)   */
#define POV_PATTERN_SPIRAL1     25   /* Spiral1Pattern::EvaluateRaw, pattern.cpp:8396  */
#define POV_PATTERN_SPIRAL2     26   /* Spiral2Pattern::EvaluateRaw, pattern.cpp:8473  */
#define POV_PATTERN_CELLS       27   /* CellsPattern::EvaluateRaw, pattern.cpp:5652    */
/* crackle: the form-weighted distances to the three nearest cell nuclei
 * (one per unit cube, placed by the same random table) under the metric,
 * plus the offset, or with `solid` the noise at the nearest nucleus; no
 * repeat.  quilted: a pigment only (its normal form is a normal function
 * of its own, normal.cpp:371-391, not built); frequency 0 by default. */
#define POV_PATTERN_CRACKLE     28   /* CracklePattern::EvaluateRaw, pattern.cpp:5760  */
#define POV_PATTERN_QUILTED     29   /* QuiltedPattern::EvaluateRaw, pattern.cpp:8067  */
#define POV_WAVE_RAMP     0       /* the default of most patterns                    */
#define POV_WAVE_SINE     1
#define POV_WAVE_TRIANGLE 2       /* the default of marble and wood                  */
#define POV_WAVE_SCALLOP  3
#define POV_WAVE_CUBIC    4
#define POV_WAVE_POLY     5
#define POV_PATTERN_MAX_ENTRIES 16
typedef struct PovGpuPattern {
    int32_t type;
    int32_t noise_generator;      /* 1 original, 2 range corrected (default), 3 Perlin */
    int32_t num_entries;          /* colour map entries (checker: its two colours)    */
    int32_t wave_type;            /* POV_WAVE_*                                       */
    double  inverse[16];          /* inverse of the pattern's TRANSFORM, row-vector form
                                     (p' = p * M), as MInvTransPoint applies it      */
    double  gradient[3];          /* gradient: the pattern's vector                  */
    /* frequency, phase, exponent, omega, lambda and agate_turb are used
       rounded to single precision, as the reference stores them (SNGL
       waveFrequency, wavePhase, waveExponent, Lambda, Omega, agateTurbScale) */
    double  frequency, phase, exponent;   /* wave modifiers (1, 0, 1 by default)     */
    double  turbulence[3];        /* classic turbulence vector                       */
    double  omega, lambda;        /* turbulence: 0.5, 2.0 by default                 */
    double  agate_turb;           /* agate_turb (1.0 by default)                     */
    int32_t octaves;              /* turbulence: 6 by default                        */
    int32_t has_turbulence;       /* the pattern has a classic turbulence warp       */
    float   values[POV_PATTERN_MAX_ENTRIES];        /* colour map values, ascending   */
    float   colours[POV_PATTERN_MAX_ENTRIES][3];    /* colour map rgb                 */
    double  brick_size[3];        /* brick: brickSize (<8, 3, 4.5> by default)       */
    double  mortar;               /* brick: mortar, single precision (SNGL)          */
    int32_t arms;                 /* spiral1 / spiral2: the number of arms           */
    int32_t crackle_solid;        /* crackle: solid                                  */
    double  crackle_form[3];      /* crackle: form (<-1, 1, 0> by default)           */
    double  crackle_metric;       /* crackle: metric (2 by default)                  */
    double  crackle_offset;       /* crackle: offset (0 by default)                  */
    double  control0, control1;   /* quilted: control0, control1 (1, 1; SNGL)        */
    /* each colour map entry's filter and transmit (TransColour): a pigment
     * with a non-zero one makes its surface transparent where the blended
     * colour filters or transmits (Post_Pigment's HAS_FILTER: the object is
     * not OPAQUE_FLAG) */
    float   filters[POV_PATTERN_MAX_ENTRIES];
    float   transmits[POV_PATTERN_MAX_ENTRIES];
} PovGpuPattern;

/* Normal perturbation (TNORMAL, source/core/material/pattern.h; applied by
 * Perturb_Normal, source/core/material/normal.cpp:784-905, from
 * ComputeLightedTexture, source/core/render/trace.cpp:812-832).  The
 * referenced pattern gives the kind (bumps, dents, wrinkles, or a continuous
 * pattern whose value the four-point slope of normal.cpp:880-902 samples),
 * the noise generator, the warps (its inverse TRANSFORM and classic
 * turbulence) and the wave; its colour map is not read.  The normal enters
 * the pattern's space through the forward TRANSFORM (Warp_Normal,
 * warp.cpp:563-580) and leaves it through the inverse (UnWarp_Normal,
 * warp.cpp:603-620).  Without a normal_map or slope_map. */
typedef struct PovGpuNormal {
    int32_t pattern;           /* 1-based index into the scene's patterns     */
    int32_t dont_scale_bumps;  /* no_bump_scale (DONT_SCALE_BUMPS_FLAG)       */
    float   amount;            /* TNORMAL::Amount, 0.5 by default             */
    float   delta;             /* TNORMAL::Delta (accuracy), 0.02 by default  */
    double  matrix[16];        /* the pattern's forward TRANSFORM, row-vector
                                  form (p' = p * M)                           */
} PovGpuNormal;

/* Light source (LightSource, source/core/scene/object.h:313) as
 * Parse_Light_Source leaves it (source/parser/parser.cpp:3345-3406):
 * `kind` says whether it is a single point or a rectangular area grid,
 * `light_type` is Light_Type (source/core/lighting/lightsource.h:78-81).
 * The light ray and its attenuation follow ComputeOneWhiteLightRay
 * (source/core/render/trace.cpp:2710-2766) and Attenuate_Light
 * (source/core/lighting/lightsource.cpp:544-612): a spotlight's cone, a
 * cylinder light's parallel beam, a parallel light's fixed direction and
 * the fade with distance.  A shadowless light casts no shadow and adds no
 * highlight (trace.cpp:1664-1714).  Area lights take the point and spot
 * types, not parallel or cylinder beams; scenes with media containers take
 * plain point lights only (the media's light intervals of spot and
 * cylinder lights, media.cpp:715-750, are not built). */
#define POV_LIGHT_POINT 0
#define POV_LIGHT_AREA  1
#define POV_LIGHT_TYPE_POINT      1   /* 0 reads as point too */
#define POV_LIGHT_TYPE_SPOT       2
#define POV_LIGHT_TYPE_SHADOWLESS 3   /* FILL_LIGHT_SOURCE */
#define POV_LIGHT_TYPE_CYLINDER   4
typedef struct PovGpuLight {
    double  center[3];
    float   colour[3];
    int32_t kind;
    double  axis1[3];
    double  axis2[3];
    int32_t area_size1;
    int32_t area_size2;
    int32_t adaptive_level;
    int32_t jitter;
    int32_t circular;
    int32_t orient;
    double  fade_distance;    /* Fade_Distance                                   */
    double  fade_power;       /* Fade_Power (0: no fade with distance)           */
    int32_t light_type;       /* POV_LIGHT_TYPE_*                                */
    int32_t parallel;         /* Parallel (a cylinder light is always parallel)  */
    double  points_at[3];     /* Points_At: the beam's direction is points_at - center */
    double  radius;           /* Radius: spot, the cosine of the hotspot angle;
                                 cylinder, the hotspot radius                    */
    double  falloff;          /* Falloff: spot, the cosine of the falloff angle;
                                 cylinder, the falloff radius                    */
    double  tightness;        /* Coeff                                           */
} PovGpuLight;

/* mesh2 data as the parser reads it: vertex_vectors, normal_vectors and the
 * face/normal index triples. */
typedef struct PovGpuMesh {
    const float*   vertices;       /* 3 * num_vertices                       */
    const float*   normals;        /* 3 * num_normals (may be NULL)          */
    const int32_t* face_indices;   /* 3 * num_triangles                      */
    const int32_t* normal_indices; /* 3 * num_triangles (NULL = flat)        */
    int32_t        num_vertices;
    int32_t        num_normals;
    int32_t        num_triangles;
    int32_t        reserved;
} PovGpuMesh;

/* Perspective camera after Parse_Camera (source/parser/parser.cpp:1335). */
typedef struct PovGpuCamera {
    double  location[3];
    double  direction[3];
    double  right[3];
    double  up[3];
    int32_t type;                  /* 0 = perspective (the only type taken) */
    int32_t reserved;
} PovGpuCamera;

/* Radiosity settings (SceneRadiositySettings, radiosity.h:139-166). */
typedef struct PovGpuRadiosity {
    int32_t enabled;
    int32_t count;
    int32_t recursion_limit;
    int32_t nearest_count;
    double  error_bound;      /* the parser's doubles (SceneRadiositySettings) */
    double  low_error_factor;
    double  gray_threshold;
    double  minimum_reuse;
    double  maximum_reuse;
    double  brightness;
    double  pretrace_start;
    double  pretrace_end;
    double  adc_bailout;
    int32_t always_sample;
    int32_t normal;
    int32_t media;
    int32_t reserved;
} PovGpuRadiosity;

/*
 * Interior media of an object (source/core/material/media.h), as the parser
 * leaves it after Media::PostProcess: coefficients per channel (extinction
 * = absorption + sc_ext * scattering), the sampling settings, constant
 * density.  scattering_type: 1 isotropic (the reference's types 1..5).
 */
typedef struct PovGpuMedia {
    int32_t scattering_type;
    int32_t method;           /* Sample_Method: 1, 2 or 3                   */
    int32_t intervals;
    int32_t min_samples, max_samples;
    int32_t aa_level;
    float   aa_threshold;
    float   jitter;
    float   absorption[3];
    float   emission[3];
    float   scattering[3];
    float   extinction[3];
    float   eccentricity;
    int32_t reserved;
} PovGpuMedia;

/*
 * Interior of an object (Interior, source/core/coretypes.h:193-215, after
 * Interior::PostProcess): what a ray entering or leaving the object through
 * a transmitting surface sees (ComputeRefraction, trace.cpp:1323-1454;
 * the fade of ComputeLightedTexture, trace.cpp:1104-1124, and of
 * ComputeShadowTexture, trace.cpp:1229-1247).  Every object of the reference
 * has one: the parser gives objects without an interior{} a default one
 * (Parser::Post_Process, parser.cpp:9225-9230), and a CSG child without its
 * own shares its parent's (parser.cpp:9040-9044).
 */
typedef struct PovGpuInterior {
    double  ior;              /* IOR (1 by default)                               */
    double  dispersion;       /* Dispersion (1 = none; the GPU path takes 1 only)  */
    double  caustics;         /* Caustics (0 = none; the GPU path takes 0 only)    */
    double  fade_distance;    /* Fade_Distance (0 = no distance attenuation)      */
    double  fade_power;       /* Fade_Power                                       */
    float   fade_colour[3];   /* Fade_Colour                                      */
    float   old_refract;      /* Old_Refract: the legacy `refraction` factor (1)  */
} PovGpuInterior;

typedef struct PovGpuSceneDesc {
    uint32_t              abi_version;   /* POV_GPU_ABI_VERSION */
    int32_t               num_objects;
    const PovGpuObject*   objects;
    int32_t               num_materials;
    const PovGpuMaterial* materials;
    int32_t               num_lights;
    const PovGpuLight*    lights;
    int32_t               num_meshes;
    const PovGpuMesh*     meshes;
    PovGpuCamera          camera;
    float                 background[4];   /* rgb + transmit             */
    float                 ambient_light[3];
    int32_t               max_trace_level;
    float                 adc_bailout;
    int32_t               language_version; /* e.g. 370                  */
    PovGpuRadiosity       radiosity;
    int32_t               num_medias;
    const struct PovGpuMedia* medias;
    int32_t               num_patterns;
    const PovGpuPattern*  patterns;
    int32_t               num_normals;
    const PovGpuNormal*   normals;
    /* interiors: object_interior[i] = 1 + index into interiors for object i,
     * 0 = the default interior (ior 1, no fade); NULL: every object has the
     * default one */
    int32_t               num_interiors;
    const PovGpuInterior* interiors;
    const int32_t*        object_interior;
    double                atmosphere_ior;   /* SceneData::atmosphereIOR (1)   */
} PovGpuSceneDesc;

/* A render block, as POVRect (inclusive bounds) plus its serial number. */
typedef struct PovGpuBlock {
    int32_t  left, top, right, bottom;
    uint32_t serial;
    uint32_t reserved;
} PovGpuBlock;

/* Render options that the view applies to every block
 * (View::StartRender, source/backend/scene/view.cpp:714-725). */
typedef struct PovGpuRenderParams {
    int32_t width;
    int32_t height;
    int32_t antialias;        /* 0 = off                                   */
    int32_t sampling_method;  /* 1 or 2 (adaptive, tracetask.cpp:604)      */
    float   aa_threshold;
    int32_t aa_depth;
    int32_t jitter;           /* 0 = off                                   */
    float   jitter_amount;
    int32_t quality;          /* +Q level, 9 = full                        */
    int32_t high_reproducibility;
} PovGpuRenderParams;

/* Counters with the reference's statistic names (statisticids.h). */
typedef struct PovGpuStats {
    uint64_t number_of_rays;        /* Number_Of_Rays: every TraceRay call  */
    uint64_t shadow_ray_tests;      /* Shadow_Ray_Tests                     */
    uint64_t shadow_rays_succeeded; /* Shadow_Rays_Succeeded                */
    uint64_t reflected_rays;        /* Reflected_Rays_Traced                */
    uint64_t number_of_pixels;      /* Number_Of_Pixels                     */
    uint64_t number_of_samples;     /* Number_Of_Samples (AA)               */
    uint64_t radiosity_gathers;     /* Radiosity samples calculated         */
    uint64_t radiosity_reuse;       /* Radiosity samples reused             */
    uint64_t device_error;          /* raw device error word (0 = none)     */
    uint64_t radiosity_rays;        /* Radiosity sample rays shot           */
    uint64_t radiosity_gathers_d0;  /* samples calculated at bounce depth 0 */
    uint64_t radiosity_gathers_d1;  /* samples calculated at bounce depth 1 */
    uint64_t nic_answers;           /* radiosity queries the neural cache answered */
    uint64_t nic_val_error_ppm;     /* its held-out relative RMSE, parts per million */
    uint64_t transmitted_rays;      /* Transmitted_Rays_Traced              */
    uint64_t media_samples;         /* Media_Samples                        */
    uint64_t refracted_rays;        /* Refracted_Rays_Traced                */
    uint64_t internal_reflected_rays; /* Internal_Reflected_Rays_Traced     */
} PovGpuStats;

/* One closest-hit result of pov_gpu_trace_rays. */
typedef struct PovGpuHit {
    int32_t object;     /* flattened object id, -1 = miss                  */
    int32_t triangle;   /* mesh triangle index, -1 for other shapes        */
    double  t;          /* hit distance along the (normalised) ray         */
} PovGpuHit;

typedef struct PovGpuScene PovGpuScene;

/*
 * Copies the scene to the current CUDA device and builds the device trees.
 * Replaces: nothing in the reference (it traces SceneData in place); called
 * where View::StartRender creates its TraceTasks
 * (source/backend/scene/view.cpp:1185-1190).  Unsupported object types,
 * textures or lights return POV_GPU_E_UNSUPPORTED and store the offending
 * object index in *bad_index (when non-NULL).
 *
 * Transparent surfaces (a plain pigment with filter or transmit, outside
 * media containers) are taken when each hit continues into one ray: no
 * reflection on a transparent material, interiors with dispersion 1 and
 * caustics 0, no media containers, radiosity or area lights in the scene,
 * the camera inside no object (*bad_index: the object around it), at most
 * 256 interiors of transparent surfaces.  A ray inside more than 7
 * interiors at once sets the device error (POV_GPU_E_DEVICE).
 */
int pov_gpu_scene_create(const PovGpuSceneDesc* desc, PovGpuScene** out, int32_t* bad_index);

/*
 * Traces whole render blocks: one call does for all blocks what
 * TraceTask::SimpleSamplingM0 (source/backend/render/tracetask.cpp:403) or,
 * with antialias on and sampling_method 2, AdaptiveSupersamplingM2
 * (tracetask.cpp:604) does per block.  out_rgbt receives 4 floats per pixel
 * in block order, each block's pixels row-major, exactly the vector that
 * CompletedRectangle takes.  out_rgbt may be host or device memory.
 * stats (optional) is overwritten with this call's counters.  It blocks
 * until the blocks are done, or returns POV_GPU_E_TIMEOUT when the scene's
 * host wait limit (pov_gpu_set_timeout) runs out first.
 */
int pov_gpu_trace_blocks(PovGpuScene* scene, const PovGpuBlock* blocks, int32_t num_blocks,
                         const PovGpuRenderParams* params, float* out_rgbt, PovGpuStats* stats);

/*
 * Closest-hit query for arbitrary rays: what Trace::FindIntersection
 * (source/core/render/trace.cpp:285, bounding method 1) returns for each
 * ray, reported as (object id, triangle, depth).  origins and directions
 * hold 3 doubles per ray; directions must be normalised.  Used for parity.
 */
int pov_gpu_trace_rays(PovGpuScene* scene, const double* origins, const double* directions,
                       int32_t num_rays, PovGpuHit* hits);

/*
 * pov_gpu_trace_rays without any device allocation.  No counterpart in the
 * reference: FindIntersection allocates nothing, and this entry gives the
 * same guarantee to callers that cannot allocate device memory --
 * integrations whose device memory is committed to another allocator (a
 * caching allocator holding the rest of HBM makes cudaMalloc fail although
 * the caller has room), and render threads sharing the GPU with frames in
 * flight, where cudaFree would synchronise the whole device.
 *
 * Same arguments and results as pov_gpu_trace_rays (objects, triangles and
 * depths are identical).  Its scratch is a fixed device array of the
 * library, 7.5 MiB per device, holding at most POV_GPU_STATIC_MAX_RAYS rays;
 * num_rays above that returns POV_GPU_E_CAPACITY and touches nothing.
 * The first call on a device does a one-time set-up (it looks up that
 * array's device address, which can make CUDA load the library's device
 * code there); make that call, e.g. with num_rays = 0, before any stream
 * capture.  The array's header (counters, error word, statistics) is zeroed
 * by every call.  There is one array per device: calls that overlap in time
 * on one device, from different threads or scenes, race on it.  The
 * array's address is looked up once per device and kept for the life of
 * the process: after cudaDeviceReset (or any teardown of the device's
 * primary context) the kept address is stale, so calls after such a reset
 * are not supported.
 */
#define POV_GPU_STATIC_MAX_RAYS 65536
int pov_gpu_trace_rays_static(PovGpuScene* scene, const double* origins, const double* directions,
                              int32_t num_rays, PovGpuHit* hits);

/*
 * Radiosity pretrace: what RadiosityTask::Run (source/backend/render/
 * radiositytask.cpp:95-263) does for the view's blocks before the final
 * render (View::StartRender, source/backend/scene/view.cpp:1056-1123):
 * empties the scene's sample cache, then traces every pretrace pass
 * (pretrace_start down to pretrace_end spacing) over the blocks, filling the
 * cache.  Call it once per frame with all blocks, before
 * pov_gpu_trace_blocks.  POV_GPU_E_INVALID when the scene has no radiosity.
 */
int pov_gpu_radiosity_pretrace(PovGpuScene* scene, const PovGpuBlock* blocks, int32_t num_blocks,
                               const PovGpuRenderParams* params, PovGpuStats* stats);

/*
 * Radiosity cache files, the reference's .rca format
 * (RadiosityCache::Load / BlockPool::Save, source/core/lighting/
 * radiosity.cpp:909-1010,1142-1170; one text line per sample as
 * ot_write_block writes it, source/core/support/octree.cpp:1345-1370).
 * pov_gpu_cache_save writes the scene's current cache (after a pretrace,
 * or after a final trace, which adds its own samples) to `path`.
 * pov_gpu_cache_load reads `path` (NULL: forget a loaded file) and makes
 * its samples the start of every following frame's cache: the cache holds
 * them at once, and each pov_gpu_radiosity_pretrace starts from them
 * instead of from an empty cache -- what +RFI does for a reference view.
 * Loaded samples have quality 1 and the file's precision (6 significant
 * digits, illuminance to 4 decimals, unit vectors packed to bytes).
 * *loaded (optional) receives the number of samples read.  Both return
 * POV_GPU_E_INVALID without radiosity or when the file cannot be opened,
 * and load returns POV_GPU_E_CAPACITY for more samples than the cache
 * holds.
 */
int pov_gpu_cache_save(PovGpuScene* scene, const char* path);
int pov_gpu_cache_load(PovGpuScene* scene, const char* path, int32_t* loaded);

/*
 * The pretrace jitter table: RadiosityTask's RandomDoubleSequence(-1, 1,
 * 2047) values (radiositytask.cpp:99), which the reference-side caller holds.
 * Copied.  Without a table the pretrace jitters by its own hash.
 */
int pov_gpu_set_pretrace_jitter(PovGpuScene* scene, const double* table, int32_t n);

/*
 * Neural irradiance cache (no reference counterpart).  When enabled, the
 * radiosity pretrace ends by training a 4x64 MLP (hand-written tcgen05
 * kernels) on the depth-0 samples it gathered, `steps` Adam steps of `batch`
 * samples; every eighth sample is held out.  If the held-out relative RMSE
 * is at most `gate` (the radiosity error_bound is the natural choice),
 * final-trace queries that no cached sample covers take the network's
 * answer instead of gathering a new sample; otherwise the plain gather
 * answers them.  Training is deterministic for given samples: each CTA
 * keeps its own gradient slice and the Adam step sums the slices in a
 * fixed order.
 */
typedef struct PovGpuNeuralCache {
    int32_t enabled;
    int32_t steps;            /* Adam steps per pretrace                      */
    int32_t batch;            /* samples per step (multiple of 128 is best);
                                 0 = 128 per SM of the device                 */
    float   learning_rate;
    float   gate;             /* largest held-out relative RMSE it may answer */
    uint32_t seed;            /* batch sampling                               */
    int32_t shared;           /* 1: one network across pretraces (views): each
                                 pretrace goes on training it from its current
                                 weights and input bounds                      */
} PovGpuNeuralCache;
int pov_gpu_set_neural_cache(PovGpuScene* scene, const PovGpuNeuralCache* config);

/*
 * The neural cache's kernels on caller data, for checking them: params holds
 * the FP32 parameter vector (POV_GPU_NIC_PARAMS floats: W1[64x112], b1[64],
 * W2[64x64], b2, W3, b3, W4, b4, W5[16x64], b5[16]; weights row-major
 * [out][in]), bounds the box (lo xyz, hi xyz) points are scaled into.
 * out (n x 3, may be NULL) receives the predictions; with targets (n x 3),
 * grad (POV_GPU_NIC_PARAMS floats) and *loss receive the gradient and value
 * of (1/n) sum (p - y)^2 / (p^2 + 0.01).  Host pointers; runs on the current
 * device.
 */
#define POV_GPU_NIC_PARAMS 20752
int pov_gpu_nic_eval(const float* params, const float* bounds, const float* points, const float* normals,
                     const float* targets, int32_t n, float* out, float* grad, float* loss);

/*
 * Host wait limit of the scene's calls, in seconds (0 = no limit, the
 * default).  A call whose queued device work has not finished when the
 * limit runs out returns POV_GPU_E_TIMEOUT instead of waiting on -- so a
 * render task can poll for stop/pause (the reference's TraceTask calls
 * Cooperate() between pixels, tracetask.cpp:403-454) -- and its outputs
 * are undefined.  The work already queued keeps running on the device and
 * still writes the scene's buffers and that call's output buffer: keep the
 * buffer alive until the next call on the scene returns (it first waits
 * for that work, within its own limit) or the scene is destroyed
 * (pov_gpu_scene_destroy waits without a limit).  POV_GPU_E_INVALID for a
 * negative or non-finite limit.
 */
int pov_gpu_set_timeout(PovGpuScene* scene, double seconds);

/* Releases all device memory of the scene (after waiting for its queued
 * work, without a limit). */
void pov_gpu_scene_destroy(PovGpuScene* scene);

/*
 * Makes the scene launch its kernels on `cuda_stream` (a cudaStream_t of the
 * scene's device; NULL = the scene's own non-blocking stream).  Lets a host
 * that owns a stream (e.g. one per View) order and time the work itself.
 * No reference counterpart: the reference has no device streams.
 */
int pov_gpu_scene_set_stream(PovGpuScene* scene, void* cuda_stream);

/*
 * Replaces the view's camera without re-parsing or rebuilding the scene:
 * the "camera changes without parsing" of View::StartRender
 * (source/backend/scene/view.cpp:862-975, render option SceneCamera).
 * `camera` holds location, direction, right and up before look_at; with
 * `look_at` non-NULL the vectors are re-aimed as that code applies look_at,
 * about `sky` (NULL = <0,1,0>).  Applies to the following trace calls; the
 * BVH, materials and lights are shared by every view.  POV_GPU_E_INVALID
 * when look_at equals the location, POV_GPU_E_UNSUPPORTED for a camera
 * inside a media container.
 */
int pov_gpu_set_camera(PovGpuScene* scene, const PovGpuCamera* camera, const double* look_at, const double* sky);

/*
 * Image output on the device: linear RGBT pixels quantised to 8 bits per
 * channel as the reference's image writers do it -- clip to [0,1], the
 * file's transfer curve, then IntEncode(gamma, x, 255) without dithering
 * (source/base/image/encoding.cpp:67-91) -- so a caller reads back 3 bytes
 * per pixel instead of 16.  `rgbt`: npix x 4 floats in device memory (e.g.
 * pov_gpu_trace_blocks' device output); `out`: npix x 3 bytes (RGB), device
 * or host memory.  Curves (source/base/image/colourspace.cpp): sRGB, the
 * default of most formats, and ITU-R BT.709, the PPM writer's.
 */
#define POV_GPU_CURVE_SRGB  0
#define POV_GPU_CURVE_BT709 1
int pov_gpu_encode_u8(PovGpuScene* scene, const float* rgbt, int64_t npix, int32_t curve, uint8_t* out);

/* Pipeline stages reported by pov_gpu_get_timings. */
#define POV_GPU_STAGE_CAMERA        0
#define POV_GPU_STAGE_TRACE_CLOSEST 1
#define POV_GPU_STAGE_SHADE         2
#define POV_GPU_STAGE_TRACE_SHADOW  3
#define POV_GPU_STAGE_RESOLVE       4
#define POV_GPU_STAGE_FINALIZE      5
#define POV_GPU_STAGE_AREA_SHADOW   6   /* area-light shadow subdivision       */
#define POV_GPU_STAGE_RADIOSITY     7   /* radiosity cache queries and gathers  */
#define POV_GPU_STAGE_MEDIA         8   /* media of rays inside containers      */
#define POV_GPU_STAGES              9

/* Profile of the last trace call.  Stage times are CUDA-event durations on
 * the launch stream, filled when profiling bit 0 is set; the work counters
 * (BVH node visits = child-box pairs tested, primitive tests, rays entering
 * each traversal kernel) when bit 1 is set.  Launch counts are always kept.
 * No reference counterpart: this is the GPU path's statistics sink, next to
 * the reference-named counters of PovGpuStats. */
typedef struct PovGpuTimings {
    float    stage_ms[POV_GPU_STAGES];
    uint32_t stage_launches[POV_GPU_STAGES];
    uint64_t node_visits[2];     /* [0] closest-hit kernels, [1] any-hit kernels */
    uint64_t prim_tests[2];
    uint64_t tri_tests[2];
    uint64_t rays_traced[2];
    uint32_t kernel_launches;    /* all kernels of the call */
    uint32_t reserved;
} PovGpuTimings;

#define POV_GPU_PROFILE_TIMES 1
#define POV_GPU_PROFILE_WORK  2
int pov_gpu_set_profiling(PovGpuScene* scene, int flags);
int pov_gpu_get_timings(PovGpuScene* scene, PovGpuTimings* out);

/*
 * Launch shapes of the trace path's kernels (no reference counterpart).
 * The project's autotuner (povray_gb300/autotune.py) times candidate
 * shapes on the device and records the best per workload in a table;
 * zero fields keep the library's defaults.  Applies to later calls.
 * POV_GPU_E_INVALID for values outside the ranges below.
 */
typedef struct PovGpuLaunchConfig {
    int32_t trace_blocks_per_sm;   /* traversal grid, blocks per SM: 1..32 (default 8)        */
    int32_t trace_block;           /* traversal block: 64 or 128 threads (default 128)       */
    int32_t trace_occupancy;       /* 1: registers capped for 8 resident blocks per SM (lean
                                      traversal of scenes without tori and CSG); 0: default */
    int32_t shade_blocks_per_sm;   /* grid cap of the queue kernels, blocks per SM: 1..64
                                      (default 16)                                           */
    int32_t bounding_tree;         /* the tree the traversal walks: 0 = the library's
                                      binned-SAH four-wide tree (default); 1 = the
                                      reference's bounding tree (Build_Bounding_Slabs /
                                      Build_BBox_Tree over the top-level objects,
                                      boundingbox.cpp:262-430,834-928, each mesh2's own
                                      tree, mesh.cpp:1376-1450, grafted under its leaf),
                                      flattened into four-wide nodes, built on first use */
    int32_t reserved[3];
} PovGpuLaunchConfig;
int pov_gpu_set_launch_config(PovGpuScene* scene, const PovGpuLaunchConfig* config);

/*
 * The traversal tree in use (no reference counterpart): its four-wide
 * nodes and levels, and -- once the reference's tree has been built -- the
 * composite nodes of the reference's top tree and of its mesh trees
 * (BBOX_TREE nodes with entries), -1 before.
 */
typedef struct PovGpuTreeInfo {
    int32_t bounding_tree;
    int32_t nodes;
    int32_t depth;
    int32_t ref_top_nodes;
    int32_t ref_mesh_nodes;
    int32_t reserved[3];
} PovGpuTreeInfo;
int pov_gpu_get_tree_info(PovGpuScene* scene, PovGpuTreeInfo* info);

/* Human-readable text of a status code. */
const char* pov_gpu_error_string(int status);

/* ABI version compiled into the library. */
int pov_gpu_abi_version(void);

#ifdef __cplusplus
}
#endif
#endif /* POVGPU_H */
