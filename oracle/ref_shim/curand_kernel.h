#pragma once
// Host stand-in for cuRAND's device API, used only to drive the reference's
// stochastic BSDF functions with EXPLICIT uniforms. Every curand_uniform()
// call pops the next value of a caller-supplied list, so a query states the
// exact random numbers the reference consumed and in which order
// (random_number_generators.h:73-92 routes all draws through curand_uniform).
struct curandStateReplay {
    const float *xs;   // caller-owned uniforms
    int n;             // number of uniforms available
    int used;          // how many curand_uniform() calls happened
};
typedef curandStateReplay curandState;
typedef curandStateReplay curandStateXORWOW_t;

inline float curand_uniform(curandState *s)
{
    float x = (s->used < s->n) ? s->xs[s->used] : 0.5f;
    s->used++;
    return x;
}
