// Host-side scene helpers shared by the procedural scenes and the glTF
// importer: the reference's host material categorisation and the default
// material record.
#pragma once
#include <cstdint>
#include "../../include/optpt.h"

namespace opthost {

// MaterialParams::isDeterministic / categorise (include/material_params.h:
// 116-223 of the reference): the host-side category of a material, or 0
// (Uncategorised) when a hit must choose its lobe stochastically.
uint32_t hostCategory(const MaterialData &m);

// A MaterialData with the given base colour, no textures (indices -1, unit
// texture-transform scales), opaque, alpha cutoff 0.5, ior 1.5, roughness 1,
// metallic 0, specular 0; category left 0.
MaterialData baseMaterial(double r, double g, double b);

}  // namespace opthost
