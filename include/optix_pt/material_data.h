/* Per-material record: the reference's MaterialData (include/material_data.h:
 * 18-60) with the same field names and meaning. The six cudaTextureObject_t
 * handles become int32 indices into the renderer's texture table (-1 = none),
 * because textures are filtered in software by the shading kernel. */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { AM_OPAQUE = 0, AM_BLEND = 1, AM_MASK = 2 }; /* include/alpha_mode.h:3-8 */

/* include/material_flags.h:3-18 */
enum {
    MF_UNCATEGORISED = 0,
    MF_METAL = 1 << 0,
    MF_DIELECTRIC = 1 << 1,
    MF_EMISSION = 1 << 2,
    MF_OPAQUE = 1 << 3,
    MF_TRANSMISSION = 1 << 4,
    MF_REFLECTION = 1 << 5,
    MF_DIFFUSE = 1 << 6,
    MF_SUBSURFACE = 1 << 7,
    MF_COAT = 1 << 8,
    MF_SHEEN = 1 << 9,
    MF_LAMBERTIAN = 1 << 10,
    MF_SPECULAR = 1 << 11
};

/* include/texture_transform.h:6-11; rotation is carried but, as in the
 * reference's shading code, not applied. */
typedef struct TextureTransform {
    float offset[2];
    float scale[2];
    float rotation;
} TextureTransform;

typedef struct MaterialData {
    int32_t baseColourTexture;
    int32_t normalTexture;
    int32_t metallicRoughnessTexture;
    int32_t emissiveTexture;
    int32_t sheenColourTexture;
    int32_t sheenRoughnessTexture;

    float baseColour[4];
    int32_t alphaMode;
    float alphaCutoff;

    float sheenColour[3];
    float emission[3];

    TextureTransform baseColourTexTf;
    TextureTransform normalTexTf;
    TextureTransform metallicRoughnessTexTf;
    TextureTransform emissiveTexTf;
    TextureTransform sheenColourTexTf;
    TextureTransform sheenRoughnessTexTf;

    float ior;
    float roughness;
    float metallic;
    float specular;
    float transmissionWeight;
    float subsurfaceWeight;
    float coatWeight;
    float coatRoughness;
    float sheenRoughness;

    uint32_t type;
    uint32_t category; /* MaterialFlags; 0 = categorised per hit */

    uint8_t hasBaseColourTexture;
    uint8_t hasNormalTexture;
    uint8_t hasMetallicRoughnessTexture;
    uint8_t hasEmissiveTexture;
    uint8_t hasSheenColourTexture;
    uint8_t hasSheenRoughnessTexture;
    uint8_t pad[2];
} MaterialData;

#ifdef __cplusplus
}
#endif
