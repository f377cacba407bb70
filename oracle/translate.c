/*
 * CPU oracle of six-frame translation — TEST INFRASTRUCTURE ONLY (see
 * oracle.h).  Restates CodonTable::translate_codes (translation.rs:277-308):
 * frame f < 3 reads codons at f, f+3, ... while a whole codon remains; frames
 * 3..5 read the reverse complement from the end (complement of code c is
 * 3 - c, codes above 3 stay), offset f - 3.  A codon with a code above 3 is X.
 */
#include "oracle.h"

static uint8_t comp(uint8_t c) { return c > 3 ? c : (uint8_t)(3 - c); }

static uint8_t codon(const uint8_t* aa64, uint8_t a, uint8_t b, uint8_t c) {
    if (a > 3 || b > 3 || c > 3) return 22; /* AA_X */
    return aa64[a * 16 + b * 4 + c];
}

size_t orc_translate_codes(const uint8_t* nt, size_t n, unsigned frame, const uint8_t* aa64, uint8_t* out) {
    size_t k = 0;
    if (frame < 3) {
        for (size_t i = frame; i + 3 <= n; i += 3) out[k++] = codon(aa64, nt[i], nt[i + 1], nt[i + 2]);
    } else {
        for (size_t j = frame - 3; j + 3 <= n; j += 3)
            out[k++] = codon(aa64, comp(nt[n - 1 - j]), comp(nt[n - 2 - j]), comp(nt[n - 3 - j]));
    }
    return k;
}
