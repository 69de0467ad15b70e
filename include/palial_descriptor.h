/*
 * palial_descriptor.h -- the tile descriptor and tile addressing of the reference, for
 * callers that do not include the reference's own include/descriptor.h.
 *
 * Layout-identical to reference include/descriptor.h:13-20 (same fields, order and types),
 * so buffers and descriptors pass unchanged between the two.  The addressing rule is the
 * reference's include/tile_address.h:9-17: tile (m,n) starts at element
 * tile_nelements * (m + (matrix_size / tile_size) * n); inside a tile, column-major, ld = NB.
 * The helpers are static inline here (the reference defines them non-static in a header
 * included by one translation unit).
 */
#ifndef PALIAL_DESCRIPTOR_H
#define PALIAL_DESCRIPTOR_H

#include <stdlib.h>

typedef struct matrix_descriptor_t {
    int tile_size;          /* NB */
    long int matrix_nelements;
    long int tile_nelements;
    int matrix_size;        /* N  */
    void *matrix;
} MATRIX_desc;

static inline MATRIX_desc palial_matrix_desc_init(int tile_size, long int matrix_nelements,
                                                  long int tile_nelements, int matrix_size)
{
    MATRIX_desc d;
    d.matrix = NULL;
    d.tile_size = tile_size;
    d.matrix_nelements = matrix_nelements;
    d.tile_nelements = tile_nelements;
    d.matrix_size = matrix_size;
    return d;
}

static inline void *palial_tile_address(MATRIX_desc A, int m, int n)
{
    size_t off = (size_t)A.tile_nelements * ((size_t)m + (size_t)(A.matrix_size / A.tile_size) * (size_t)n);
    return (void *)((double *)A.matrix + off);
}

#endif
