/*
 * shadytracer.h -- the C ABI of the GB300 rendering hot path (libshadytracer.so).
 *
 * Plain C types only: no CUDA, no C++ and no torch types cross this boundary, so a JavaScript host
 * (an N-API addon), Python (ctypes) or C can bind it. Every call returns an int status: 0 (ST_OK) or
 * a negative ST_ERR_* code; st_last_error() says why in words. No C++ exception crosses it.
 *
 * What each entry point replaces in the reference (lampmaker/ShadyTracer v0.88.0, paths relative to
 * its root):
 *   st_create / st_destroy       createPathTracer + RT.init / RT.dispose      lib/pathtracer/index.js:90,
 *                                                                             core/raytrace_main.js:121,1291
 *   st_set_scene                 RT.setScene(scene) (the scene contract)      lib/pathtracer/index.js (setScene),
 *                                                                             core/raytrace_main.js:1145,
 *                                                                             lib/pathtracer/README.md:126-145
 *   st_set_params                RT.set(values) -> unknown keys               lib/pathtracer/README.md:56,
 *                                                                             core/uniforms.schema.js (UniformSpec)
 *   st_set_view                  the camera uniforms genrays reads            core/genrays.js:65-92
 *   st_invalidate                RT.invalidate()                              lib/pathtracer/README.md:38-124
 *   st_step / st_step_async /    RT.step(n) (resolves when the GPU finished)  lib/pathtracer/index.js:1005,
 *   st_sync                                                                   core/raytrace_main.js:1574 (R.trace)
 *   st_read_accum                the accumulation + error-bar moments read    core/wavefront.js:414-494 (prog_resolve),
 *                                                                             core/measure.js:36-66
 *   st_image_stats               R.imageStats()                               core/raytrace_main.js:876-950
 *   st_read_counters             the Counters struct readback                    core/wavefront.js:150
 *   st_kernel_times              per-kernel GPU time (kerneltime.js)          core/kerneltime.js:1-25
 *   st_sppm_*                    the photon map's store / grid / gather       core/sppm.js:305-511
 *   st_optics_*                  createOptics(RT, WG): O.setSources/setFar/run optics/index.js:92,434-475,
 *                                                                             optics/kernels.js:288-408,571-699
 *   st_last_error                the JS exception's message                   core/raytrace_main.js:1580-1581
 *
 * Threading: one CUDA stream per context; a context is not thread-safe (the JS host is single-threaded).
 * Memory: caller-owned output buffers; the library owns its device memory.
 */
#ifndef SHADYTRACER_H
#define SHADYTRACER_H

#ifndef __CUDACC_RTC__                 /* NVRTC (a scene's code, compiled at st_set_scene) has the types built in */
#include <stddef.h>
#include <stdint.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define ST_ABI_VERSION 1

/* status codes */
#define ST_OK            0
#define ST_ERR_ARG      -1   /* a bad argument: null pointer, size out of range, unknown enum */
#define ST_ERR_OOM      -2   /* device memory could not be allocated */
#define ST_ERR_CUDA     -3   /* a CUDA call failed (no device, launch failure) */
#define ST_ERR_TIMEOUT  -4   /* st_sync ran out of time, or a device-side wait ran out of iterations */
#define ST_ERR_BUSY     -5   /* a trace is in flight (st_step_async without st_sync) */
#define ST_ERR_COMPILE  -6   /* a scene failed to build; the previous scene is kept */
#define ST_ERR_STATE    -7   /* called in the wrong state (no scene, no view) */

typedef struct st_ctx st_ctx;

/* ---------------------------------------------------------------------------------------------
 * THE SCENE, AS DATA: a table of primitives folded the way the reference's scene prelude folds a
 * scene (core/scene_api.js:28-80 add_new / fold): each item is one primitive, or a CSG chain of them
 * (smooth union / union / subtraction into the item before), and the items are folded by the nearest
 * surface (argmin |d|), the medium being the least-deep item the point is inside.
 * --------------------------------------------------------------------------------------------- */
enum st_prim_type {
    ST_PRIM_PLANE    = 0,  /* z = 0 in the local frame, +z out                                     */
    ST_PRIM_SPHERE   = 1,  /* p0 radius                                              sdf.js:217     */
    ST_PRIM_BOX      = 2,  /* p0..p2 half sizes                                       sdf.js:220    */
    ST_PRIM_ROUNDBOX = 3,  /* p0..p2 half sizes, p3 rounding                          sdf.js:224    */
    ST_PRIM_TORUS    = 4,  /* p0 ring radius R, p1 tube radius r (xy plane)           sdf.js:602    */
    ST_PRIM_PRISM    = 5,  /* p0 sides, p1 corner radius, p2 height (z), p3 rounding  shapes.js:266-287 */
    ST_PRIM_ASPHERE  = 6,  /* p0 D, p1 t, p2 R1, p3 k1, p4 a4_1, p5 a6_1, p6 R2, p7 k2, p8 a4_2, p9 a6_2
                                                                                      shapes.js:621-660 */
    ST_PRIM_CYLINDER = 7   /* p0 half height (z), p1 radius                           sdf.js:228    */
};
enum st_prim_op {
    ST_OP_ITEM   = 0,      /* starts a new fold item                                               */
    ST_OP_SMOOTH = 1,      /* smooth union into the current item, radius k            sdf.js:252    */
    ST_OP_UNION  = 2,      /* hard union into the current item                                     */
    ST_OP_SUB    = 3       /* subtracted from the current item                                     */
};

/* 128 bytes, 16-byte aligned fields: staged whole into shared memory by a bulk copy. */
typedef struct st_prim {
    uint32_t type, op, material, flags;  /* flags: bit 0 = emits a detector tag (optics), reserved  */
    float    pos[3];                     /* centre, metres                                          */
    float    k;                          /* smooth-union radius, metres (ST_OP_SMOOTH)               */
    float    rot[9];                     /* world -> local rotation, row major                      */
    float    pad0[3];
    float    p[12];                      /* shape parameters (st_prim_type)                          */
} st_prim;

/* A material: the fields of the reference's Material2 (core/materials.js:12-60) the hot path reads. */
typedef struct st_material {
    float base[3];        /* baseColor                                                            */
    float metallic;
    float roughness;      /* perceptual; alpha = roughness^2, delta below alpha 1e-3               */
    float specular;       /* 0.5 = the physical interface, 0 = no coat                            */
    float specular_tint;
    float transmission;
    float ior;
    float abbe;           /* Abbe number V_d; 0 = not dispersive (spectral.js cauchyN)             */
    float attenuation;    /* attenuationDistance (m); 0 = tint at each crossing                    */
    float detector;       /* optics: > 0.5 stops and records a ray (optics/kernels.js optIsDetector)*/
    float emissive[3];    /* cd/m^2                                                               */
    float beam_cos;       /* an emitter's beam (builder/lights.js beamShape, the cone of a cosine light): > 0,
                           * the cosine of its half angle -- the emission, emissive straight out, only within that
                           * cone about the surface's outward normal; 0, a glowing surface, the same every way   */
    float haze;           /* of what transmission passes, the share diffused through rather than refracted
                           * (materials.js Material2.haze): 0 clear, 1 an opal face                              */
    float anisotropy;     /* stretches the gloss along the surface's first tangent: 0 round, 1 ten to one
                           * (materials.js Material2.anisotropy; the frame the normal's own, no grain)           */
    /* A COATING (materials.js:52-89 Material2.coat, coatR, coatEdge, coatWidth, coatIndex; :150-163 coatMaterial):
     * a thin-film stack that is the interface instead of the bare Fresnel. R(lambda) runs from coat_lo below
     * coat_edge (nm, at normal incidence) to coat_hi above it, a logistic of 10-90 % width coat_width (nm, 0 a step);
     * the edge moves to shorter wavelengths with the angle through the stack's effective index coat_index. A
     * channel's reflectance is R averaged over that channel's wavelengths. coat: where it is -- 0 none, 1 on the
     * faces light enters by with the faces it leaves by anti-reflective, 2 entering with the leaving faces bare
     * (the glass's Fresnel), 3 every face. On a metal the stack lies over it. specular and specular_tint do nothing
     * where a coating is. coat_lo and coat_hi are held to [0, 1], coat_width to >= 0, coat_index to >= 1. */
    uint32_t coat;
    float coat_lo, coat_hi;
    float coat_edge;      /* nm                                                                     */
    float coat_width;     /* nm                                                                     */
    float coat_index;
    /* SCATTER INSIDE (materials.js:102-111 scatterDistance, scatterAnisotropy; haze.js:574-650 the medium's walk): the
     * mean free path between scatterings in the material's volume (metres; 0 a clear volume) and the Henyey-Greenstein
     * asymmetry of each scattering (held to +-0.95). A ray that refracts into the material walks it: free flights
     * drawn from exp(-d / scatter_distance), each collision turning it by the phase function and weighing 1; the
     * colour and the loss stay attenuation's, over the whole walk. */
    float scatter_distance;
    float scatter_g;
    float pad[2];         /* 112 bytes                                                              */
} st_material;

/* A LIGHT'S FACE (builder/lights.js, the builder's light object; core/scene_api.js:259-289 LightFace,
 * lightFaceArea, lightFaceDensity): a one-sided rectangle or disc of luminance le straight out along
 * n = u x v, in a beam (lights.js:209-228 beamOf / beamShape). The library draws it -- a sheet of its
 * material appended to the primitives, as the builder's codegen draws a light -- and light sampling
 * aims at a point uniform on it (materials_pbr.js:1244-1268; haze.js:324-350 from the air), half the
 * light samples of a vertex going to the faces; a BSDF's hit of it is weighed against that density.
 * A face is never discovered as an emitter. 80 bytes. */
enum st_light_shape { ST_LIGHT_DISC = 1, ST_LIGHT_RECTANGLE = 2 };
enum st_light_dist  { ST_LIGHT_COSINE = 0, ST_LIGHT_UNIFORM = 1 };
typedef struct st_light {
    float    centre[3];    /* metres                                                               */
    uint32_t shape;        /* st_light_shape                                                       */
    float    u[3];         /* the face's first axis (unit); a rectangle's width runs along it        */
    float    half_w;       /* half the width, or the disc's radius, metres                          */
    float    v[3];         /* the second axis (unit, at right angles to u); the face emits along u x v */
    float    half_h;       /* half the height (a rectangle), metres                                */
    float    le[3];        /* luminance straight out, cd/m^2 (lights.js fluxFactor: flux = le A k)   */
    uint32_t material;     /* the face's material: what the march meets there (no emission of its own) */
    uint32_t dist;         /* st_light_dist: cos^n intensity (radiance cos^(n-1)), or even intensity  */
    float    n;            /* the cos^n exponent (1: Lambertian)                                    */
    float    beam_cos;     /* the cosine of the beam's half angle (0: 90 degrees)                   */
    uint32_t pad;
} st_light;
#define ST_MAX_LIGHTS 64

typedef struct st_scene_desc {
    const st_prim*     prims;
    uint32_t           n_prims;        /* at most ST_MAX_PRIMS                                      */
    const st_material* materials;
    uint32_t           n_materials;    /* at most ST_MAX_MATERIALS; material 0 is the air           */
    float              env_radius;     /* metres; where the scene stops (photometry.js:158)         */
    float              tolerance;      /* metres; 0 = the automatic 1 mm (photometry.js:141-150)    */
    /* THE HAZE BOX (core/haze.js:64-80 hazeUniforms), metres; sigma_t 0 = none */
    float              haze_centre[3];
    float              haze_sigma_t;   /* 1 / mean free path, per metre                            */
    float              haze_axes[9];   /* the box's unit axes, rows                                */
    float              haze_half[3];
    float              haze_albedo[3];
    float              haze_g;         /* Henyey-Greenstein asymmetry, |g| <= 0.95                  */
    const st_light*    lights;         /* the lights' faces, or NULL                                */
    uint32_t           n_lights;       /* at most ST_MAX_LIGHTS; n_prims + n_lights <= ST_MAX_PRIMS */
} st_scene_desc;

#define ST_MAX_PRIMS      256
#define ST_MAX_MATERIALS  256

/* ---------------------------------------------------------------------------------------------
 * THE SETTINGS the hot path reads (core/uniforms.schema.js UniformSpec; their derived uniforms are
 * computed on the host in double precision, as core/photometry.js:182-237 derive() does).
 * --------------------------------------------------------------------------------------------- */
typedef struct st_params {
    uint32_t width, height;       /* the picture                                                   */
    uint32_t maxbounce;           /* 10                                                            */
    uint32_t maxiter;             /* 400: march steps a path may take in all                       */
    float    stepscale;           /* 0.9                                                           */
    uint32_t nee;                 /* 1: next-event estimation                                      */
    uint32_t rr;                  /* 0: Russian roulette after 3 bounces                           */
    float    nee_sun_pick;        /* 0.5: share of light samples sent at the sun's cone            */
    float    sun_elevation;       /* degrees                                                       */
    float    sun_azimuth;         /* degrees                                                       */
    float    sun_diameter;        /* degrees (0.53)                                                */
    float    sun_illuminance;     /* lux at normal incidence (the disc's)                           */
    float    sky_luminance;       /* cd/m^2 of the uniform sky above the horizon                    */
    float    ground_luminance;    /* cd/m^2 below the horizon                                      */
    float    env_uniform;         /* > 0: the white-furnace environment, this luminance everywhere  */
    float    env_sun_gain;        /* 1                                                             */
    float    env_sky_gain;        /* 1                                                             */
    uint32_t sun_hint;            /* 1: the sun's cone is sampled                                  */
    uint32_t seed;                /* base seed of the sample sequence                              */
    uint32_t maxaverages;         /* 0: a true mean; N: an EMA window of N                          */
    float    eps;                 /* surface tolerance setting, metres; 0 = the scene's             */
    uint32_t budget;              /* wavefront iterations a sample runs; 0 = the worst case,
                                     maxbounce + 1 + ceil(maxiter / 32) (raytrace_main.js:1815)   */
    uint32_t samples_per_wave;    /* 0 = automatic                                                 */
    /* the photon map (core/sppm.js): sun photons traced through glass and mirrors before each sample's
     * camera rays, stored where they first land on an evaluable surface, gathered by camera rays that
     * have seen only glass and mirrors since the eye; one sample a wave while it runs */
    uint32_t sppm;                /* 1 on                                                           */
    uint32_t sppm_photons;        /* photons a sample (0: one a pixel)                              */
    float    sppm_r1;             /* the first sample's radius, metres (0: 5 mm)                    */
    float    sppm_alpha;          /* the radius schedule's alpha (0: 2/3)                           */
    float    sppm_half;           /* the sun photons' square, half width, metres (0: min(15, radius)) */
    uint32_t sppm_learn;          /* 1: the sun's photons drawn from the learned 128^2 emission map
                                   * (wavefront.js:628-711), rebuilt every 4 samples from each cell's
                                   * stores per photon sent, mixed with a 20 % uniform floor; 0: uniform */
    /* the learned proposal (no counterpart in the reference, which removed its path guiding): a network of the
     * surface point (hash-grid position, harmonics of the normal; 3 x 64 hidden, BF16 on the tensor cores) gives a
     * mixture of 8 von Mises-Fisher lobes that a camera path's BSDF sampling is mixed with under one-sample MIS at its
     * evaluable opaque vertices; trained online on the incident light the paths find, between waves */
    uint32_t guide;               /* 1 on                                                           */
    float    guide_alpha;         /* the mixture's share of the one-sample MIS (0: 0.5)             */
    float    guide_lr;            /* Adam's learning rate (0: 0.005)                                 */
    uint32_t guide_train;         /* 1: train after every wave; 0: the weights as they are          */
    uint32_t guide_seed;          /* the initial weights' seed (a change draws them afresh)          */
    /* emissive surfaces (materials_pbr.js:887-960, wavefront.js:715-815): camera paths that meet an emitter
     * discover it; every 2 samples the discovered emitters become a list of bounding spheres that light sampling
     * aims at (under MIS with the BSDF's hits of them) */
    float    emit_share;          /* the light samples' share aimed at the list once it holds any (0: 0.5; clamped
                                   * to [0.05, 0.95]; the reference's neeEmitShare)                   */
    float    emit_radius;         /* the discovery grid's half-size, metres (0: 15; capped at the scene's radius)  */
    uint32_t emit_off;            /* 1: no light sampling of emitters (discovery goes on)            */
    uint32_t env_map_off;         /* 1: light sampling does not draw from the environment image's map  */
    /* THE STEP CACHE (core/wavefront.js:67-150 stepCacheWGSL, prog_stepcache_fill): a grid over the bounded
     * primitives' box, each cell the scene's distance at its centre -- a ball with no surface in it, which a ray
     * inside it may cross to where it leaves with no distance evaluation, when that is at least a cell */
    uint32_t step_cache;          /* 0 off, 1 the ray's own cell, 2 also the two cells ahead              */
    float    step_cache_cells;    /* cells, millions (0.25..16; 0: 4)                                     */
    /* LIGHT TRACING TO THE CAMERA (materials_pbr.js:672-830 ltConnect, wavefront.js:1292-1310, :1649-1661): the
     * sun's photons, traced through glass and mirrors, connect to the camera where they first land on a surface in air
     * that a connection can evaluate -- a shadow ray to the camera (through the thin lens at a point of its disc), and
     * what reaches it is added to its pixel as it is, not averaged with the pixel's paths. The camera's paths then
     * leave the class light -> delta+ -> D -> eye to the photons (a first vertex drawn from an evaluable lobe, delta
     * events after it, the sun's disc where the photons' square covers the line); with the photon map on too, the
     * map gathers only past delta events from the eye, as the reference splits the two. One sample a wave. */
    uint32_t lt;                  /* 1 on (the reference's photoncount > 0)                          */
    uint32_t lt_photons;          /* photons a sample with the photon map off (0: one a pixel); with it on, its
                                   * sppm_photons serve both, and sppm_half is the photons' square either way */
    /* THE ENVIRONMENT'S PRESETS (core/environment.js, the reference's environment as code with its presets' text):
     * ST_ENV_ANALYTIC the disc of sun_illuminance in a uniform sky (sky_luminance above the horizon, ground_luminance
     * below); ST_ENV_SUNSKY the sun and sky physically (SUNSKY_FN): sunlight of sun_outside lux above the atmosphere, a
     * 5778 K white, through air (Rayleigh), aerosol (Mie, Henyey-Greenstein 0.7, albedo 0.9) and ozone in 16 bands of
     * the spectrum, the disc what the air lets through and the sky that light scattered once toward the eye;
     * ST_ENV_STUDIO an even light brighter above (STUDIO_FN), no sun. The two presets are baked into the map light
     * sampling draws half its environment samples from, as an image is (an image, st_set_env_image, replaces all). */
    uint32_t env_mode;
    float    sun_outside;         /* ST_ENV_SUNSKY: lx above the atmosphere (0: 128 000)             */
    float    sky_turbidity;       /* ST_ENV_SUNSKY: the aerosol's depth at 550 nm is 0.05 + 0.1 x this (0.7 a clear day) */
    float    studio_illuminance;  /* ST_ENV_STUDIO: lx on a level surface facing up                   */
    float    studio_top;          /* ST_ENV_STUDIO: 0 even, 1 none from straight below (L0 (1 + top z)) */
    float    studio_color[3];     /* ST_ENV_STUDIO: its colour (normalised to luminance 1)             */
    /* LIGHT TRACING'S EMITTER PHOTONS (wavefront.js:552-588 probes, tracebasics.js:726-831 THE PROBE): with light
     * tracing on in a scene with emissive materials, this share of a sample's photons (all of them with the sun off)
     * are probes -- a listed emitter box by its probability, a random line through its bounding sphere, followed from
     * the far end back; at the first emissive surface seen from outside a probe becomes a photon leaving along the line,
     * its flux the emission over the probes and the line density there (Crofton) -- which then connect and are stored
     * as the sun's are; the camera's paths leave the emitters' light in light tracing's class to them */
    float    lt_emit_share;       /* 0: 0.5; clamped to [0.05, 0.95] while the sun shines (the reference's ltEmitShare) */
    /* THE ENVIRONMENT IN A TEXTURE (core/envmap.js, UniformSpec envCache / envCacheSize, on by default there): a
     * preset's light baked once a change into an equirectangular env_cache_size x half texture (2 x 2 points a texel,
     * the sun's cone left out), which every ray that leaves and every light sample reads bilinearly; in the sun's cone
     * the preset itself is asked */
    uint32_t env_cache;           /* 1 on                                                           */
    uint32_t env_cache_size;      /* 1024, 2048 or 4096 (0: 2048)                                  */
    /* THE PHOTON MAP IN THE VOLUME (sppm.js:497-511 sppmGatherVolume, haze.js mediumStore): with the map on in a scene
     * with a material that scatters inside, the sun's photons store a record where they collide inside it (past a
     * delta event, as at a surface), and a camera ray that came in through delta events alone gathers at its first
     * collision sum p(l . v) Phi / (sigma_s 4/3 pi R^3) / n^2 over the records within R, then walks on. R is the
     * first sample's volume radius shrunk as a volume: R_k^3 = R_1^3 prod_{i<k} (i + alpha) / (i + 1). */
    float    sppm_r1_volume;      /* metres (0: 4 x the surface's first radius)                       */
} st_params;

#define ST_ENV_ANALYTIC 0u
#define ST_ENV_SUNSKY   1u
#define ST_ENV_STUDIO   2u

/* The camera, as genrays reads it (core/genrays.js:65-92): the basis from invView's columns and the
 * two diagonal entries of invProjection. */
typedef struct st_view {
    float    cam_pos[3];
    float    right[3];
    float    up[3];
    float    fwd[3];              /* from the target to the camera: the view looks down -fwd         */
    float    fx, fy;              /* invProjection[0][0], [1][1]: tan(fov/2) * aspect, tan(fov/2)    */
    uint32_t camtype;             /* 0 perspective, 1 orthographic                                 */
    float    lens_radius;         /* the thin lens's aperture radius, metres (camLens.x; 0: a pinhole) */
    float    focus_distance;      /* the distance to the plane in focus along -fwd, metres (camLens.y) */
} st_view;

typedef struct st_counters_t {
    uint64_t paths;               /* camera paths deposited                                        */
    uint64_t segments;            /* path segments marched                                         */
    uint64_t march_steps;         /* SDF evaluations of the march                                  */
    uint64_t shadow_rays;         /* shadow rays traced                                            */
    uint64_t shadow_steps;        /* SDF evaluations of the occlusion pass                         */
    uint32_t nonfinite;           /* deposits refused (NaN, inf, negative luminance)               */
    uint32_t flushed;             /* paths the last iteration had to end                           */
    uint32_t shadowcut;           /* shadow rays out of steps                                      */
    uint32_t samples;             /* samples folded since the last invalidate                      */
    uint64_t launches;            /* kernels the wave chains ran (graph nodes counted) since st_create */
    /* the march's fold, counted only in a counting pass (st_enable_kernel_times(ctx, 2)): primitive
     * evaluations by type (ST_PRIM_*) and the warp instructions that issued them; bounding-sphere tests
     * and their warp issues. Their ratios are the fold's SIMD efficiency. */
    uint64_t prim_evals[8];
    uint64_t prim_warp_evals[8];
    uint64_t bound_tests;
    uint64_t bound_warp_tests;
    uint64_t op_evals[4];         /* the evaluations by how they fold in (ST_OP_*; ITEM: a chain's head) */
} st_counters_t;

typedef struct st_image_stats_t {
    double mean_luma;             /* over sampled pixels                                           */
    double median_luma;
    double trimmed_mean_luma;     /* the middle 98 %                                               */
    double mean_rel_se;           /* mean of se / L over pixels with L > 0                          */
    uint32_t sampled;             /* pixels with a sample                                          */
    uint32_t samples;             /* samples folded                                                */
} st_image_stats_t;

typedef struct st_kernel_time {
    char     name[24];
    uint32_t launches;
    double   ms;                  /* summed CUDA-event time on the context's stream                 */
} st_kernel_time;

/* ---- life cycle ---- */
int  st_create(int device, st_ctx** out);
int  st_destroy(st_ctx* ctx);
/* ctx NULL: why the calling thread's last st_render_noalloc was refused ("no context" if it was not) */
const char* st_last_error(const st_ctx* ctx);
int  st_abi_version(void);

/* ---- the scene, the settings, the camera ---- */
/* THE SCENE, AS DATA OR AS CODE (the reference's scene contract, lib/pathtracer/README.md:126-145: its `wgsl` is the
 * scene's SDF and material functions, builder/codegen.js:974-1060 generates them; setScene compiles them,
 * core/raytrace_main.js:1145). cuda_src NULL: the scene is desc's primitive table, folded by a loop over it.
 * cuda_src given: CUDA C++ that defines, at file scope over the library's device types,
 *     __device__ float        st_scene_dist(st::f3 p);      the signed distance at p (FOLD_DIST)
 *     __device__ st::SceneHit st_scene_full(st::f3 p);      distance, material of the nearest surface, medium (FOLD_FULL)
 * (and, with #define ST_SCENE_COUNTS, __device__ float st_scene_dist_count(st::f3 p, uint32_t* wc), the distance
 * tallying its work with st::wc_prim / st::wc_test for the counting pass); it is compiled by NVRTC for sm_103a with
 * the kernels that ask the scene and loaded (a source compiled before in the process is taken from a cache). desc
 * still gives the materials, the haze, the lights' faces and the radii; its primitives, which may then be none,
 * bound the space sort and the step cache and are what the optics trace folds. shadytracer_gb300/codegen.py writes
 * such code from a table or a node tree. On failure -- a bad table, or code that does not compile (ST_ERR_COMPILE;
 * errbuf holds NVRTC's log, each error followed by the scene's line it names) -- the previous scene is kept. */
int  st_set_scene(st_ctx* ctx, const char* cuda_src, const st_scene_desc* desc, char* errbuf, size_t errlen);
/* the scene in force: is_code 1 when it was given as code; NVRTC's time for it (0 when it came from the cache) and its
 * cubin's size */
int  st_scene_code_info(st_ctx* ctx, int* is_code, double* compile_ms, uint64_t* cubin_bytes);
/* a scene's code compiled for sm_103a into the process's cache, with no device or context (the builder's check that a
 * scene compiles before it is set): ST_OK, or ST_ERR_COMPILE with NVRTC's log in errbuf as st_set_scene gives it;
 * compile_ms NVRTC's time (0 when the source was compiled before). A later st_set_scene of the same source loads it. */
int  st_compile_scene(const char* cuda_src, char* errbuf, size_t errlen, double* compile_ms);
/* unknown_mask: reserved (0); the struct has no unknown keys. Changing the picture size or the
 * settings resets the accumulation. */
int  st_set_params(st_ctx* ctx, const st_params* p, uint64_t* unknown_mask);
int  st_set_view(st_ctx* ctx, const st_view* v);
/* MANY VIEWS IN ONE WAVEFRONT (the batching of many views in one persistent launch): n cameras of the same scene and
 * settings (1..ST_MAX_VIEWS), each a picture of its own, rendered together -- every step a sample of each, their paths
 * in the same waves, one march and one occlusion pass over all of them, one photon pass shared. A view's paths take
 * the random numbers the same view rendered alone takes, so each picture is the one st_set_view would give (but for
 * the order of f32 deposits into a pixel, and what discovery and training gather from all the views together). Light
 * tracing connects to one camera: st_step refuses it with more than one view. st_set_view is st_set_views(ctx, v, 1). */
#define ST_MAX_VIEWS 16
int  st_set_views(st_ctx* ctx, const st_view* views, uint32_t n);
/* a view's picture, as st_read_accum reads view 0's */
int  st_read_accum_view(st_ctx* ctx, uint32_t view, double* rgb, double* V, double* S, uint32_t* count);
/* THE ENVIRONMENT IMAGE (core/envimage.js, the image preset of core/environment.js; core/envmap.js the map light
 * sampling draws from): an equirectangular panorama, w x h pixels of linear rgb floats, top row first, its middle
 * column +x, running right as one turns right, turned turn_deg about z (anticlockwise from above); luminance is the
 * cd/m^2 of a unit (0: 179, a Radiance file's efficacy). It becomes the whole environment -- no sun, sky or ground --
 * and light sampling draws half its environment samples from a 512 x 256 equal-area map of it (envMapShare), baked on
 * the GPU here. rgb NULL goes back to the sun and sky. Resets the accumulation. */
int  st_set_env_image(st_ctx* ctx, const float* rgb, uint32_t w, uint32_t h, float luminance, float turn_deg);
/* The map's tables from its texels' mean luminances (envmap.js:215-260 envSampling), host-only: lum 512 x 256 floats,
 * rows from straight up; tex 512 x 256 x 4 floats (the CDF along the row at the texel's end, the density per
 * steradian, the CDF down the rows at the row's end, 0). Returns 0, or ST_ERR_ARG. */
int  st_env_map_tables(const float* lum, float* tex);
int  st_invalidate(st_ctx* ctx);

/* ---- tracing ---- */
int  st_step(st_ctx* ctx, int n);             /* n samples; returns when the GPU has finished       */
int  st_step_async(st_ctx* ctx, int n);       /* queue n samples                                    */
int  st_sync(st_ctx* ctx, int timeout_ms);    /* wait for the queued samples; <0 waits forever      */
/* THE DEVICE-SIDE WAITS (the guard the reference keeps on the host: core/wavefront.js:298-303 clamps an indirect
 * dispatch that could run forever, core/raytrace_main.js:67 cuts a frame's submissions short): every kernel that stages
 * a table into shared memory waits for its copy at most `iterations` times (0: the default, 2^24), then flags the
 * error and returns; st_sync then reports ST_ERR_TIMEOUT once (the flag is cleared) and the context stays usable --
 * st_invalidate before trusting the picture again. arm_only 1 is the test of that path: the waits are armed but no
 * copy is issued, so each runs out at its limit with nothing in flight. Kept until changed. */
int  st_set_wait_limit(st_ctx* ctx, uint32_t iterations, int arm_only);
/* THE AUTOTUNER (the batching's tile sizes and march-step caps, picked on the workload itself): each pair of the march's
 * and the occlusion pass's queue tile -- the entries a warp claims at a time, 32, 64 or 128 -- and march chunk -- the
 * scene evaluations a ray takes a launch before it waits for the next iteration, 24 to 160 -- timed over `samples`
 * samples of the scene, settings and view in force; the fastest is kept for the renders that follow and returned, with
 * its time and the defaults' (64, 48). The accumulation is cleared. The picture does not depend on either. */
typedef struct st_tune {
    uint32_t claim;               /* queue entries a warp claims at a time (0: 64)                   */
    uint32_t chunk;               /* evaluations a ray takes a launch (0: 48)                        */
    float    ms;                  /* the pick's time for the tuning samples                           */
    float    ms_default;          /* the defaults' time                                               */
} st_tune;
int  st_autotune(st_ctx* ctx, int samples, st_tune* out);
int  st_set_tune(st_ctx* ctx, const st_tune* t);    /* set them (claim, chunk; 0 the defaults)       */

/* ---- readings (caller-owned buffers, width*height entries each; NULL skips one) ---- */
int  st_read_accum(st_ctx* ctx, double* rgb, double* V, double* S, uint32_t* count);
/* CHECKPOINT AND RESUME: the render's state between samples as one blob -- the FP64 accumulation of every view (mean
 * rgb and count), the error bar's moments, light tracing's splat buffer and connection counts, and the sample index the
 * next samples are seeded by. Loaded into a context with the same scene, settings and picture (after st_sync, before
 * its next step), the render goes on where it stopped: the samples after it take the random numbers they would have
 * taken, so a render saved at N samples and resumed to N + M is the one rendered to N + M at once. What learns across
 * samples is the caller's to carry (the proposal's weights, st_mlp_get_weights / st_mlp_set_weights); the emitters'
 * list and the learned emission map start over. The blob is st_checkpoint_size's bytes; a load of another picture's
 * blob (its width, height or views) is ST_ERR_ARG. */
int  st_checkpoint_size(st_ctx* ctx, size_t* bytes);
int  st_checkpoint_save(st_ctx* ctx, void* out, size_t bytes);
int  st_checkpoint_load(st_ctx* ctx, const void* in, size_t bytes);
int  st_image_stats(st_ctx* ctx, st_image_stats_t* out);
int  st_read_counters(st_ctx* ctx, st_counters_t* out);
/* The scene's signed distance at n points (3n floats, metres) into out (n floats), as the march folds the table
 * (scene_api.js FOLD_DIST, each primitive behind its bounding-sphere test). */
int  st_eval_sdf(st_ctx* ctx, const float* pts, uint32_t n, float* out);
/* Per-kernel GPU time, CUDA events on the context's stream around every launch while enabled (launches then
 * run directly rather than as a replayed graph). on = 2 also counts the march's fold work into the counters
 * (a counting pass: an instrumented march, so its times are not the plain kernel's). */
int  st_enable_kernel_times(st_ctx* ctx, int on);
int  st_kernel_times(st_ctx* ctx, st_kernel_time* out, int max, int* n_out);
int  st_reset_kernel_times(st_ctx* ctx);
/* The microfacet albedo tables the context built at init (microfacet.js:245-330): 16*32*32 Ec,
 * 16*32 Ec_avg, 32*32 E1 floats. */
int  st_mf_tables(st_ctx* ctx, float* ec, float* ecavg, float* e1);

/* ---- the photon map (core/sppm.js) ----
 * Records are SoA: pos (3 floats), power (3), the direction it came from and its surface normal as
 * octahedral words, bounce|flags|sub word. st_sppm_build sorts n records into the grid of cell size
 * `cell` (metres) over 2^20 hashed cells by a counting sort; st_sppm_read_grid returns each record's
 * hash (key), the per-cell counts and the cell-ordered record permutation. */
typedef struct st_sppm_stats {
    uint32_t stored;              /* records in the grid                                           */
    uint32_t gathers;             /* gathers run                                                   */
    uint32_t cut;                 /* gathers that reached the hard cap (the wavefront's map: records dropped) */
    uint32_t visits_max;          /* most records one gather looked at                              */
    uint64_t visits;              /* records looked at in all                                      */
} st_sppm_stats;

int  st_sppm_build(st_ctx* ctx, const float* pos, const float* power, const uint32_t* dir_oct,
                   const uint32_t* nrm_oct, const uint32_t* flags, uint32_t n, float cell);
int  st_sppm_read_grid(st_ctx* ctx, uint32_t* key, uint32_t* cell_count, uint32_t* cell_start,
                       uint32_t* order);
/* gather at m query points: pos (3m), normal (3m), the surface's albedo (3m; Lambertian f = albedo/pi) and the
 * camera path's bounces at each; out (3m, FP64) = sum f * power over the records within `radius` (at most half the
 * cell) on a facing surface inside the bounce cap (core/sppm.js:305-346,475-494); budget: records a gather may walk
 * (0 = unlimited; past a cell's share of it, sub-lists), seed: the sub-lists' draws. */
int  st_sppm_gather(st_ctx* ctx, const float* qpos, const float* qnrm, const float* qalbedo,
                    const uint32_t* qbounce, uint32_t m, float radius, uint32_t maxbounce,
                    uint32_t budget, uint32_t seed, double* out);
int  st_sppm_stats_read(st_ctx* ctx, st_sppm_stats* out);
/* THE LEARNED EMISSION MAP (st_params.sppm_learn; core/wavefront.js:628-711 ltEmit / ltHit / ltCdf, prog_lt_build), as
 * the last sample left it: per cell of the 128 x 128 square the sun's photons cross, the photons sent through it and
 * those stored (128^2 each, halved at every rebuild), and the CDF they are drawn from (128^2 conditional row entries,
 * then 128 rows). NULL skips one. ST_ERR_STATE before the photon map has run. */
int  st_sppm_emission_map(st_ctx* ctx, uint32_t* sent, uint32_t* stored, float* cdf);
/* LIGHT TRACING'S MAP OF CONNECTIONS (st_params.lt; the splat buffer's fourth word, wavefront.js:1656-1660): per pixel
 * (W x H) the photons' connections that reached the camera since the last invalidate -- where light tracing lights
 * the picture, and how densely. ST_ERR_STATE before a wave has run. */
int  st_lt_counts(st_ctx* ctx, uint32_t* counts);

/* ---- the optics bench (optics/index.js, optics/kernels.js) ---- */
typedef struct st_optics_source {
    float    centre[3];           /* metres                                                        */
    float    flux;                /* lm: its share of the rays follows it                          */
    float    axis[3];             /* emission axis, unit                                           */
    uint32_t shape;               /* 0 point, 1 disc, 2 rectangle, 3 a ray set (st_optics_set_rays) */
    float    tangent[3];          /* first tangent                                                 */
    float    size_x;              /* disc radius / rectangle half width                            */
    float    size_y;              /* rectangle half height                                          */
    uint32_t dist;                /* 0 collimated, 1 uniform cone, 2 cos^n                          */
    float    cos_half;            /* cos of the cone's half angle                                   */
    float    n_exp;               /* the cos^n exponent (1: Lambertian)                             */
    float    emit_n;              /* the index it emits into                                        */
    uint32_t two_sided;
    uint32_t on_surface;          /* start 2 march tolerances off the sheet                          */
    uint32_t instance;            /* which instance of a batch it belongs to                        */
    uint32_t ray_first, ray_count;/* a ray set's rays in the ray table: each traced ray takes one at
                                     random, as it is, carrying its weight (kernels.js:320-336)       */
    /* THE LIGHT'S COLOUR (builder/sources.js colour, planck, spectrum; optics/spectral.js sourceSpectrum): its rays
     * carry this linear Rec.709 colour at the flux's luminance (0, 0, 0: white). The trace by wavelength
     * (st_optics_batch.spectral) draws them from its spectrum: row `spectrum` - 1 of st_optics_set_spectra's table when
     * set, else a blackbody of `cct` kelvin when set, else a stand-in spectrum of exactly the colour's XYZ. */
    float    colour[3];
    float    cct;
    uint32_t spectrum;
    uint32_t pad[5];              /* 128 bytes                                                      */
} st_optics_source;

typedef struct st_optics_far {
    uint32_t nC, nG;              /* type C grid: nC about the axis, nG from 0 to 180 degrees       */
    float    axis[3];             /* gamma = 0                                                      */
    float    c0[3];               /* C = 0, square to the axis                                      */
} st_optics_far;

/* A batch of independent instances traced in one launch chain: instance i owns rays
 * [ray_first[i], ray_first[i] + ray_count[i]) and the scene items whose st_prim.flags >> 8 == i, which
 * must be contiguous in the table; an item naming an instance past the batch is an error. */
typedef struct st_optics_batch {
    uint32_t n_instances;
    const uint32_t* ray_count;    /* rays per instance                                             */
    uint32_t lux_cells;           /* the lux map is lux_cells^2 per instance (0 none)               */
    float    lux_half;            /* its half width, metres                                         */
    float    lux_height;          /* its distance from the source along the axis, metres            */
    uint32_t maxbounce;           /* 0 = 32                                                         */
    uint32_t seed;
    /* THE TRACE BY WAVELENGTH (optics/spectral.js, the scene's `spectral` feature): 1 -- each ray carries three
     * wavelengths of its light's spectrum, drawn stratified through x-bar + y-bar + z-bar (u, u + 1/3, u + 2/3), a
     * weight each S(l) / (3 p(l)); a material's colour is a reflectance at each (sum_c rgb_c B_c(l), B the clipped
     * Rec.709 colour-matching functions over their sum), a coating its R at each, and a dispersive glass refracts
     * the first and drops the other two (the ray's weights become 3 w_1, 0, 0); tallies count Y = sum_k w_k y-bar(l_k)
     * and the detector's hits its X and Z. 0: the rays carry a colour, as the renderer's do. */
    uint32_t spectral;
} st_optics_batch;

typedef struct st_optics_totals {
    double   emitted;             /* weight emitted (rays)                                          */
    double   escaped, lost, detected, absorbed;   /* weight                                         */
    uint64_t interactions;
    uint64_t rays;
    uint64_t n_escaped, n_lost, n_detected, n_absorbed;   /* rays (optics/kernels.js O_COUNT)     */
} st_optics_totals;

/* WHAT A RUN KEEPS BEYOND ITS TALLIES (optics/kernels.js:174-251): the detector hits (optRecordHit) up to det_cap, and
 * the paths of each instance's first path_rays rays (optVertex) up to path_verts vertices each, an escaped ray's last
 * esc_len (metres) past its last interaction. All 0: nothing kept (the default). */
typedef struct st_optics_detail {
    uint32_t det_cap;             /* detector hits kept a run (at most 2^24)                        */
    uint32_t path_rays;           /* rays an instance whose paths are kept (at most 4096)          */
    uint32_t path_verts;          /* vertices a kept path (at most 256)                            */
    float    esc_len;             /* metres (0: 0.1)                                                */
} st_optics_detail;

int  st_optics_set_sources(st_ctx* ctx, const st_optics_source* src, uint32_t n);
int  st_optics_set_far(st_ctx* ctx, const st_optics_far* far);
/* THE RAY TABLE the ray sets read (optics/sources.js RAYSET_VEC4; a Zemax source file's rays placed by the host,
 * optics/zemax.js): n rays of 8 floats -- position (metres, world), weight (its flux over its set's mean),
 * direction (unit), wavelength (nm, 0 none). */
int  st_optics_set_rays(st_ctx* ctx, const float* rays, uint32_t n);
/* THE SPECTRA a source may name (st_optics_source.spectrum): n rows of ST_SPECTRUM_NODES values, a spectral power
 * distribution at 1 nm from ST_SPECTRUM_LO nm (any scale: each is normalised to luminance 1), replacing the table. */
#define ST_SPECTRUM_LO    360
#define ST_SPECTRUM_NODES 471
int  st_optics_set_spectra(st_ctx* ctx, const float* values, uint32_t n);
/* Traces every instance of the batch; far (n_instances*nG*nC) and lux (n_instances*cells^2) are the
 * FP64 tallies in ray weight (the host multiplies by flux / rays); totals per instance. */
int  st_optics_run(st_ctx* ctx, const st_optics_batch* batch, double* far, double* lux,
                   st_optics_totals* totals);
int  st_optics_set_detail(st_ctx* ctx, const st_optics_detail* detail);
/* the optics autotuner: the batch run with each queue tile and march chunk of st_autotune's candidates, the fastest
 * kept for the runs that follow (st_tune as st_autotune returns it); the tallies are the last run's */
int  st_optics_autotune(st_ctx* ctx, const st_optics_batch* batch, st_tune* out);
/* THE LAST RUN'S TALLIES BY OBJECT AND BY MATERIAL (optics/kernels.js:651-681, O_TAG and O_MAT): per tag -- an item
 * of the table, by its first primitive's index, 256 of them -- and per (instance, material) the weight incident, the
 * weight leaving and the interactions, 3 doubles each; tags 256 x 3, mats n_instances x n_materials x 3 (NULL skips) */
int  st_optics_tallies(st_ctx* ctx, double* tags, double* mats);
/* THE LAST RUN'S DETECTOR HITS: n_out the hits that reached a detector (past det_cap only the first det_cap kept), up
 * to max_n of them into hits, 12 floats each: position (metres), weight, direction, tag (the item's first primitive),
 * instance, CIE X and Z of its colour (Y the weight), 0 */
int  st_optics_hits(st_ctx* ctx, float* hits, uint32_t max_n, uint32_t* n_out);
/* THE LAST RUN'S KEPT PATHS: counts (n_instances x path_rays) their vertices, verts (n_instances x path_rays x
 * path_verts x 8 floats) each vertex's position, weight, optical length and hue rgb (the ray's colour at luminance 1) */
int  st_optics_paths(st_ctx* ctx, float* verts, uint32_t* counts);

/* ---- the learned proposal (st_params.guide) ----
 * The parameters, FP32, in one array of ST_MLP_PARAMS: W1 (64 x 48), W2 (64 x 64), W3 (64 x 64), W4 (40 x 64), each
 * [out][in] row-major, then the hash grid's features (16 levels x 2^12 entries x 2). Inputs: 2 features a level of a
 * trilinear blend over the box's cells (level l has floor(2 * 16^(l/15)) cells across the box's longest side), then
 * the 16 real spherical harmonics of degree <= 3 of the normal; outputs: 8 lobes x (mean direction, unnormalised;
 * log kappa, clamped to [-1, 6]; mixture logit). */
#define ST_MLP_PARAMS (13824u + 131072u)
typedef struct st_mlp_stats {
    uint32_t steps;               /* Adam steps since the weights were set                          */
    uint32_t samples;             /* training samples in the last wave's batch                      */
    float    loss;                /* the last wave's loss a sample                                  */
    float    mean_weight;         /* the last batch's mean weight (f cos L_in / pdf at the vertex)   */
    float    box_lo[3];           /* the hash grid's box: its low corner, metres                     */
    float    box_inv_ext;         /* ... and 1 / its longest side                                    */
    uint32_t inferred;            /* vertices the network ran at in the last wave                   */
} st_mlp_stats;
int  st_mlp_get_weights(st_ctx* ctx, float* out, size_t n);
int  st_mlp_set_weights(st_ctx* ctx, const float* in, size_t n);
/* the network at n points (pos, nrm: 3n): raw (40n) its outputs; mix (40n) each lobe's mean direction, kappa and
 * weight as the sampler reads them (quantised: the mean direction in 2 x 16 bits, kappa and the weight as halves) */
int  st_mlp_eval(st_ctx* ctx, const float* pos, const float* nrm, uint32_t n, float* raw, float* mix);
/* the gradient (ST_MLP_PARAMS) of sum_i -(w_i / mean w) log q(dir_i | pos_i, nrm_i), each normalised weight capped
 * at 20, with respect to every parameter, at 1 to 16384 samples, without a step; loss: the sum */
int  st_mlp_grad(st_ctx* ctx, const float* pos, const float* nrm, const float* dir, const float* weight, uint32_t n,
                 float* grad, float* loss);
/* `steps` training steps (Adam, learning rate lr; 0: 0.005) on the given batch of 1 to 131072 samples, mini-batches of
 * 16384 in turn: what a wave's end does with the records its paths made */
int  st_mlp_train(st_ctx* ctx, const float* pos, const float* nrm, const float* dir, const float* weight, uint32_t n,
                  uint32_t steps, float lr);
int  st_mlp_stats_read(st_ctx* ctx, st_mlp_stats* out);
/* the last wave's training batch, at most max_n samples of 10 floats (position, normal, direction, weight) */
int  st_mlp_read_batch(st_ctx* ctx, float* out, uint32_t max_n, uint32_t* n);

/* ---- emissive surfaces ----
 * The list light sampling aims at, as the last build left it: per box its bounding sphere's centre and radius
 * (metres), its probability and the running sum of the probabilities (6 floats a box, in the grid's voxel order). */
int  st_emit_list(st_ctx* ctx, float* out, uint32_t max_n, uint32_t* n);

/* ---- a render that allocates nothing ----
 * No counterpart in the reference: an entry point for hosts that may not allocate device memory when they want a
 * picture -- one held to a memory budget fixed at start-up, one on a real-time thread, one whose allocations would
 * land inside a stream capture it does not own. It renders `nsamples` samples of a picture of at most 128 x 128
 * pixels (ST_NOALLOC_MAX_PIXELS) into the caller's host buffers (width*height entries each; NULL skips one), using
 * only a scratch array compiled into the library: 8 MiB (ST_NOALLOC_SCRATCH_BYTES) of device memory on every GPU that
 * loads the library, held until exit. No cudaMalloc, no cudaFree, no allocating library call. A larger picture, or
 * more than 256 primitives or materials, returns ST_ERR_ARG. Each call clears the accumulation and counters it keeps
 * in the shared array and runs on the device's legacy default stream; calls that overlap on one GPU race, so a host
 * serialises them. The first call on a device does the set-up (the array's address, the albedo tables) and should
 * come before any stream capture. The caller's current device is as it was when the call returns. The result equals
 * st_step's for the same inputs. What this render does not carry is refused with ST_ERR_ARG, and
 * st_last_error(NULL) says why: light faces, st_params.sppm, st_params.lt, st_params.guide, st_params.step_cache,
 * st_params.env_mode other than ST_ENV_ANALYTIC, and an emissive
 * material unless st_params.emit_off is set (then both paths render it by the BSDF's hits alone). */
#define ST_NOALLOC_MAX_PIXELS (128u * 128u)
#define ST_NOALLOC_SCRATCH_BYTES (8u << 20)
int  st_render_noalloc(int device, const st_scene_desc* desc, const st_params* p, const st_view* v, int nsamples,
                       double* rgb, double* V, double* S, uint32_t* count);

/* ---- the binding's checks ---- */
/* The sizes of the structs above as this library was built (st_prim, st_material, st_scene_desc, st_params,
 * st_view, st_counters_t, st_image_stats_t, st_kernel_time, st_sppm_stats, st_optics_source, st_optics_far,
 * st_optics_batch, st_optics_totals, st_mlp_stats, st_light, st_optics_detail, st_tune, in that order); returns how many
 * it has. */
int  st_struct_sizes(uint32_t* out, int max);
/* The context's CUDA stream (a cudaStream_t), for a host that orders or times its own work against it. */
void* st_stream(st_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* SHADYTRACER_H */
