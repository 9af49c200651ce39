#pragma once
// Host stand-in for the OptiX SDK header. The reference's BSDF and sampling
// headers include <optix.h> only for the OptixTraversableHandle typedef that
// LaunchParams carries; none of the BSDF arithmetic uses OptiX.
typedef unsigned long long OptixTraversableHandle;
