// Two-run 16-bit column layout ("duo" records) of the mixed solver's FP32
// matrix copy, in the matrix's own numbering (host-side construction, once
// per sparsity pattern).
//
// A row's sorted columns are split at their largest gap into two runs; each
// run gets a 32-bit base and each column a 16-bit offset from it:
//     col = (e < split ? base1 : base2) + off        (e = entry index in the row)
// which fits whenever both runs span at most 65535 columns.  That holds for
// the vertex-then-entity numberings of P1 / P2 spaces on meshes numbered
// plane by plane, whose rows touch one window of the vertex block and one
// window of the entity block.  Entries are grouped in pairs (a row of odd
// length gets a padding entry: value 0, offset 0 from base2, a column of the
// row): the two values as a float2, the two offsets as one 32-bit word, so a
// lane reads two entries with two loads -- 6 instead of 8 bytes per entry.
// Per row one int4 record {first duo, base1, base2, split | duos << 16}.
#pragma once
#include <cstdint>
#include <vector>

struct DuoLayout {
    int n = 0;
    int64_t nduo = 0;
    int max_span = 0;               // largest run span over all rows
    std::vector<int32_t> meta;      // [4 * (n + 1)] per row {first duo, base1, base2, split | duos << 16};
                                    // row n holds the total duo count in its first word
    std::vector<uint32_t> off;      // [nduo] two 16-bit offsets (entry 2d in the low half)
    std::vector<int32_t> src;       // [nduo] CSR position of the duo's first entry; -1 - position when the
                                    // second entry is padding
};

// Builds the layout from the CSR pattern (columns ascending per row).
// Returns 0, or 1 when a run spans more than 65535 columns, a row has more
// than 65535 entries or the duo count exceeds 32-bit indexing (the layout is
// then not usable).
int duo_build(int n, const int32_t *rowptr, const int32_t *cols, DuoLayout *L);
