/* rt_oracle.h — TEST INFRASTRUCTURE ONLY: C API of the scalar CPU oracle.
 *
 * Loaded with ctypes by tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline leg. Parity against the reference is unpinned (the reference
 * has no implementation of this path); see oracle_common.hpp.
 * Ray / hit records use the layouts of include/fnd_rt.h (32 B / 8 B). */
#ifndef RT_ORACLE_H
#define RT_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_bvh orc_bvh;

orc_bvh* orc_bvh_build(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, uint32_t bins,
                       uint32_t max_leaf);
void orc_bvh_free(orc_bvh* b);
/* out[0]=nodes out[1]=leaves out[2]=depth out[3]=largest leaf; *sah = normalised SAH cost */
void orc_bvh_stats(const orc_bvh* b, uint64_t* out, double* sah);
/* 0 when every triangle is in exactly one leaf, leaves hold <= max_leaf
 * triangles and every box encloses its children / triangles */
int orc_bvh_validate(const orc_bvh* b);
float orc_bvh_margin(const orc_bvh* b);

/* stats[0] = binary node boxes fetched, stats[1] = triangle tests (may be NULL) */
void orc_trace_closest(const orc_bvh* b, const void* rays, uint64_t n, void* hits, uint32_t threads,
                       uint64_t* stats);
void orc_trace_any(const orc_bvh* b, const void* rays, uint64_t n, uint8_t* out, uint32_t threads,
                   uint64_t* stats);
void orc_brute_closest(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, const void* rays,
                       uint64_t n, void* hits, uint32_t threads);
void orc_brute_any(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, const void* rays,
                   uint64_t n, uint8_t* out, uint32_t threads);
/* one ray (8 floats) against one triangle (9 floats): returns hit flag;
 * out5 = t, U, V, W, det */
int orc_intersect1(const float* ray8, const float* v9, float* out5);
void orc_pcg32_fill(uint64_t seed, uint64_t seq, uint32_t* out, uint64_t n);
double orc_time_build_ms(const float* verts, uint32_t nv, const uint32_t* idx, uint32_t nt, uint32_t bins,
                         uint32_t max_leaf);

#ifdef __cplusplus
}
#endif
#endif
