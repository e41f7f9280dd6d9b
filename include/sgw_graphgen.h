/*
 * sgw_graphgen.h — seeded synthetic graph generators and graph utilities.
 *
 * The reference ships only a text-to-binary converter (tools/converter.cpp)
 * and reads real graphs from disk.  These functions build the synthetic
 * inputs the engine is measured on, in memory, deterministically from a
 * seed, in the same CSR layout as a .bcsr/.bwcsr file.
 *
 * Random numbers: SplitMix64 (Steele, Lea and Flood, "Fast splittable
 * pseudorandom number generators", OOPSLA 2014), indexed by edge number so
 * the output does not depend on the thread count.
 */
#ifndef SGW_GRAPHGEN_H
#define SGW_GRAPHGEN_H

#include "subway_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* R-MAT (Chakrabarti, Zhan and Faloutsos, SDM 2004): 2^scale vertices,
 * edge_factor * 2^scale directed edges drawn by recursive quadrant choice
 * with probabilities (a, b, c, 1-a-b-c) and no vertex permutation (vertex 0
 * is the top hub).  Self-loops and duplicate edges are removed, rows are
 * sorted by destination, and the out-edges of vertex n-2 are dropped so that
 * graphs read by the reference's loader (which never writes outDegree[n-2],
 * shared/graph.cu:179-181) mean the same thing there as here.
 * Weighted graphs get w = 1 + (hash(seed, src, dst) mod wmax).
 * Fails with SGW_ERANGE if the edge count after deduplication reaches 2^32
 * (the u32 header of the binary format, shared/graph.cu:43-44). */
int sgw_gen_rmat(uint32_t scale, uint32_t edge_factor, double a, double b,
                 double c, uint64_t seed, int weighted, uint32_t wmax,
                 sgw_graph **out);

/* Erdos-Renyi G(n, m) control: m uniform (src, dst) pairs, same cleaning. */
int sgw_gen_er(uint32_t n, uint64_t m, uint64_t seed, int weighted,
               uint32_t wmax, sgw_graph **out);

/* Adds every reverse edge (weight kept) and removes duplicates: the
 * symmetrised input CC is run on. */
int sgw_graph_symmetrize(const sgw_graph *g, sgw_graph **out);

/* Picks count sources uniformly (seeded) among the vertices of the largest
 * weakly connected component that have out-degree > 0. */
int sgw_pick_sources(const sgw_graph *g, uint32_t count, uint64_t seed,
                     uint32_t *out);

/* Vertices and edges of the largest weakly connected component. */
int sgw_largest_wcc(const sgw_graph *g, uint32_t *vertices, uint64_t *edges);

#ifdef __cplusplus
}
#endif
#endif /* SGW_GRAPHGEN_H */
