#pragma once
struct curandState { unsigned long long s; };
inline void curand_init(unsigned long long seed, unsigned long long, unsigned long long, curandState *st) { st->s = seed; }
inline float curand_uniform(curandState *st) { st->s = st->s * 6364136223846793005ULL + 1442695040888963407ULL; return (float)((st->s >> 40) & 0xFFFFFF) / 16777216.0f; }
