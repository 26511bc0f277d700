/*
 * gpm_gen.h — seeded synthetic data graphs and host CSR utilities.
 *
 * The reference reads its data graphs from text files
 * (DataLoader::general_load_data, src/dataloader.cpp:20-163).  The
 * benchmark graphs here are generated instead, deterministically from a seed
 * (the same CSR on every machine and thread count): R-MAT and Chung-Lu.
 * Every CSR is symmetric, sorted, without self loops or duplicate edges.
 * Arrays are malloc'ed by the library and released with gpm_free.
 */
#ifndef GPM_GEN_H
#define GPM_GEN_H

#include "gpm.h"

#ifdef __cplusplus
extern "C" {
#endif

/* R-MAT with 2^scale vertices and edge_factor * 2^scale draws, quadrant
 * probabilities (a, b, c, 1-a-b-c). */
GPM_API int gpm_gen_rmat(int32_t scale, int32_t edge_factor, double a, double b, double c, uint64_t seed,
                         uint32_t** rowptr, int32_t** col, int32_t* v_cnt);

/* Chung-Lu power-law graph: n vertices, expected weights proportional to
 * (i+1)^(-1/(gamma-1)) scaled to an average degree of avg_degree and capped at
 * max_degree (<= 0: no cap); round(n*avg_degree/2) endpoint-pair draws. */
GPM_API int gpm_gen_chung_lu(int32_t n, double avg_degree, double gamma, int32_t max_degree, uint64_t seed,
                             uint32_t** rowptr, int32_t** col, int32_t* v_cnt);

/* Symmetric CSR from m undirected edges (src[i], dst[i]); self loops and
 * duplicates dropped.  Replaces the sort/unique/offset steps of
 * src/dataloader.cpp:129-160. */
GPM_API int gpm_csr_from_edges(int32_t v_cnt, int64_t m, const int32_t* src, const int32_t* dst,
                               uint32_t** rowptr, int32_t** col);

/* Host copy renumbered by descending degree, ties by id (the reference's
 * oriented_type 1, src/dataloader.cpp:96-109). */
GPM_API int gpm_csr_relabel_degree(int32_t v_cnt, const uint32_t* rowptr, const int32_t* col,
                                   uint32_t** rowptr_out, int32_t** col_out);

GPM_API void gpm_free(void* p);

#ifdef __cplusplus
}
#endif

#endif /* GPM_GEN_H */
