/*
 * cf_types.h — buffer records shared by the clustered-forward light-culling
 * library, its kernels and its host callers.
 *
 * Every record is byte-identical to the record the HelloVulkan clustered
 * forward pipeline already binds, so an engine hands its own buffers (or
 * copies of them) to this library without repacking:
 *
 *   CfLightData          <-> LightData         Shaders/LightData.glsl:1-6 (std430,
 *                                              array stride 48) and
 *                                              Header/Resources/ResourcesLight.h:13-21
 *   CfAABB               <-> AABB              Shaders/AABB/AABB.glsl:1-5,
 *                                              Header/Resources/ResourcesLight.h:24-30
 *   CfLightCell          <-> LightCell         Shaders/ClusteredForward/Header.glsl:1-5,
 *                                              Header/Resources/ResourcesLight.h:33-39
 *   CfClusterForwardUBO  <-> ClusterForwardUBO Shaders/ClusteredForward/Header.glsl:7-19
 *                                              (std140), Header/UBOs.h:67-89 (C++ sizeof 176)
 *
 * Matrices are column-major, element (col, row) at [col * 4 + row], as GLSL
 * and glm store them.
 *
 * Plain C99 / C++ / CUDA; no dependencies beyond <stdint.h>.
 */
#ifndef CF_TYPES_H
#define CF_TYPES_H

#include <stdint.h>

#if defined(__cplusplus)
#define CF_ALIGNAS(n) alignas(n)
#else
#define CF_ALIGNAS(n) _Alignas(n)
#endif

/* Per-cluster light cap of the reference (Header/Configs.h:55,
 * Shaders/ClusteredForward/LightCulling.comp:17). */
#define CF_MAX_LIGHTS_PER_CLUSTER_DEFAULT 150u

/* Default grid of the reference (Header/Configs.h:49-52). */
#define CF_SLICE_COUNT_X_DEFAULT 16u
#define CF_SLICE_COUNT_Y_DEFAULT 9u
#define CF_SLICE_COUNT_Z_DEFAULT 24u

/* One point light, std430 array element: position (w = 1) @0, color @16,
 * radius @32, padded to a 48-byte stride. */
typedef struct CfLightData {
    CF_ALIGNAS(16) float position[4];
    float color[4];
    float radius;
    float _pad[3];
} CfLightData;

/* One cluster's view-space bounding box; w is 0 in both points. */
typedef struct CfAABB {
    CF_ALIGNAS(16) float minPoint[4];
    float maxPoint[4];
} CfAABB;

/* Where a cluster's light indices live in the index list. */
typedef struct CfLightCell {
    uint32_t offset;
    uint32_t count;
} CfLightCell;

/* Circular motion of one light in the horizontal plane, advanced one frame
 * at a time on the device (cf_animate_light_orbits): offset' = R * offset
 * with R = [[cos, -sin], [sin, cos]] the rotation of one frame (omega * dt),
 * then position = (center.x + offset.x, center.y, center.z + offset.z,
 * center.w).  No reference counterpart: the reference's lights are static
 * (ResourcesLight::UpdateLightPosition, Source/Resources/ResourcesLight.cpp:20-29,
 * moves one light from the host). */
typedef struct CfLightOrbit {
    CF_ALIGNAS(16) float offset[2]; /* (x, z) from the centre              */
    float rot[2];                   /* (cos, sin) of the angle per frame   */
    float center[4];                /* x, y, z and the position's w        */
} CfLightOrbit;

/* What Scene.frag's cluster lookup (Shaders/ClusteredForward/Scene.frag:54-78)
 * finds for one fragment, and how its light list serves it (cf_lookup_clusters). */
typedef struct CfFragmentSample {
    uint32_t cluster;   /* clusterIdx; 0xFFFFFFFF when the lookup leaves the grid     */
    uint32_t offset;    /* lightCells[clusterIdx].offset                              */
    uint32_t count;     /* lightCells[clusterIdx].count                               */
    uint32_t covering;  /* lights of the list whose sphere contains the fragment      */
    uint32_t missing;   /* (all-lights check) lights NOT in the list that contain it  */
    uint32_t flags;     /* CF_FRAGMENT_* bits                                         */
    float view_z;       /* the fragment's view-space z, from its depth                */
    float linear_depth; /* LinearDepth(gl_FragCoord.z, near, far)                     */
} CfFragmentSample;

#define CF_FRAGMENT_OUTSIDE_GRID 1u  /* zIndex (or x, y) beyond the grid: no cluster */
#define CF_FRAGMENT_OUTSIDE_AABB 2u  /* the fragment lies outside its cluster's box   */
#define CF_FRAGMENT_CAPPED 4u        /* the cluster's list holds the cap of lights     */
#define CF_FRAGMENT_BAD_CELL 8u      /* the cell points outside the index list, or an
                                        index is not a light: nothing read through it */

/* The PBR push constants of the clustered-forward fragment pass, byte for
 * byte (Shaders/PBR/PBRPushConstants.glsl:1-8, Header/PushConstants.h:22-29). */
typedef struct CfPBRPushConstant {
    float lightIntensity;
    float baseReflectivity;
    float maxReflectionLod;
    float lightFalloff;
    float albedoMultipler;
} CfPBRPushConstant;

/* One G-buffer texel for cf_shade_clusters: the inputs Scene.frag gathers per
 * fragment (world position and window depth, the shading normal, linear
 * albedo, metallic and roughness). */
typedef struct CfGBufferTexel {
    CF_ALIGNAS(16) float position[4]; /* world xyz, w = gl_FragCoord.z (0..1) */
    float normal[4];                  /* unit normal xyz, w = metallic        */
    float albedo[4];                  /* linear albedo rgb, w = roughness     */
} CfGBufferTexel;

/* The frustum of FrustumCulling.comp, byte for byte (Shaders/Frustum.glsl:1-5,
 * Header/UBOs.h:91-98): six planes (left, right, bottom, top, near, far) as
 * rows of projection * view, and the eight corners of the clip cube
 * unprojected to world space. */
typedef struct CfFrustum {
    CF_ALIGNAS(16) float planes[6][4];
    float corners[8][4];
} CfFrustum;

/* VkDrawIndirectCommand (Shaders/DrawIndirectCommand.glsl:1-7). */
typedef struct CfDrawIndirectCommand {
    uint32_t vertexCount;
    uint32_t instanceCount;
    uint32_t firstVertex;
    uint32_t firstInstance;
} CfDrawIndirectCommand;

/* Per-view parameters, std140: invProj @0, view @64, screenSize @128,
 * sliceScaling @136, sliceBias @140, near @144, far @148, X/Y/Z @152/156/160.
 * 164 bytes are used; the C++ mirror in the reference is 176 bytes. */
typedef struct CfClusterForwardUBO {
    CF_ALIGNAS(16) float cameraInverseProjection[16];
    float cameraView[16];
    float screenSize[2];
    float sliceScaling;
    float sliceBias;
    float cameraNear;
    float cameraFar;
    uint32_t sliceCountX;
    uint32_t sliceCountY;
    uint32_t sliceCountZ;
    uint32_t _pad[3];
} CfClusterForwardUBO;

#if defined(__cplusplus)
#include <cstddef>
static_assert(alignof(CfLightData) == 16 && alignof(CfAABB) == 16 && alignof(CfClusterForwardUBO) == 16,
              "16-byte aligned records");
static_assert(sizeof(CfLightData) == 48, "LightData std430 stride is 48");
static_assert(offsetof(CfLightData, position) == 0, "LightData.position @0");
static_assert(offsetof(CfLightData, color) == 16, "LightData.color @16");
static_assert(offsetof(CfLightData, radius) == 32, "LightData.radius @32");
static_assert(sizeof(CfAABB) == 32, "AABB is two vec4");
static_assert(offsetof(CfAABB, maxPoint) == 16, "AABB.maxPoint @16");
static_assert(sizeof(CfLightCell) == 8, "LightCell is two uint");
static_assert(offsetof(CfLightCell, count) == 4, "LightCell.count @4");
static_assert(sizeof(CfClusterForwardUBO) == 176, "ClusterForwardUBO C++ sizeof");
static_assert(sizeof(CfLightOrbit) == 32 && offsetof(CfLightOrbit, center) == 16, "LightOrbit is two float4");
static_assert(sizeof(CfFragmentSample) == 32, "FragmentSample is 32 bytes");
static_assert(sizeof(CfPBRPushConstant) == 20, "PBRPushConstant is five floats");
static_assert(sizeof(CfFrustum) == 224 && offsetof(CfFrustum, corners) == 96, "FrustumUBO layout");
static_assert(sizeof(CfDrawIndirectCommand) == 16, "VkDrawIndirectCommand is four uint");
static_assert(sizeof(CfGBufferTexel) == 48, "GBufferTexel is three float4");
static_assert(offsetof(CfClusterForwardUBO, cameraView) == 64, "view @64");
static_assert(offsetof(CfClusterForwardUBO, screenSize) == 128, "screenSize @128");
static_assert(offsetof(CfClusterForwardUBO, sliceScaling) == 136, "sliceScaling @136");
static_assert(offsetof(CfClusterForwardUBO, sliceBias) == 140, "sliceBias @140");
static_assert(offsetof(CfClusterForwardUBO, cameraNear) == 144, "near @144");
static_assert(offsetof(CfClusterForwardUBO, cameraFar) == 148, "far @148");
static_assert(offsetof(CfClusterForwardUBO, sliceCountX) == 152, "X @152");
static_assert(offsetof(CfClusterForwardUBO, sliceCountY) == 156, "Y @156");
static_assert(offsetof(CfClusterForwardUBO, sliceCountZ) == 160, "Z @160");
#endif

#endif /* CF_TYPES_H */
