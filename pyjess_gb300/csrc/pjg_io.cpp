// pjg_io.cpp — native PDB atom-record reader (host code of libpjg).
//
// Structure ingestion in front of the search: the PDB reader of the
// reference's Python layer (src/pyjess/_io.py:52-103, PDBMoleculeParser)
// feeds Atom_parse, one fixed-column ATOM/HETATM record at a time.  This
// reader scans a whole PDB text in one call and writes the atom records in
// the 59-byte packed row layout of the package's atom table (the NumPy
// ATOM_DTYPE of pyjess_gb300/_records.py), so loading thousands of files
// costs no per-atom Python work.  It takes the plain forms PDB files use
// (decimal integers and reals in their columns, printable ASCII); any other
// form makes it stop and report the line, and the caller parses the text
// with its general reader instead, so both paths give the same records.

#include <cstdint>
#include <cstring>

#include "../../include/pjg.h"

namespace {

// Row layout (offsets in bytes, little endian, no padding).
constexpr int ROW = 59;
constexpr int O_X = 0, O_OCC = 24, O_TEMP = 28, O_SERIAL = 32, O_NAME = 36, O_ALT = 40, O_RES = 41, O_CHAIN = 45,
              O_RESSEQ = 47, O_ICODE = 51, O_SEG = 52, O_ELEM = 56, O_CHARGE = 58;

inline bool is_space(char c) { return c == ' ' || c == '\t'; }

// Trim [b, e) of spaces and tabs.
inline void trim(const char *&b, const char *&e) {
    while (b < e && is_space(*b)) b++;
    while (e > b && is_space(e[-1])) e--;
}

// A decimal integer field: optional sign, digits.  Empty -> `empty`.
bool parse_int(const char *b, const char *e, int64_t empty, int64_t *out) {
    trim(b, e);
    if (b == e) {
        *out = empty;
        return true;
    }
    bool neg = false;
    if (*b == '+' || *b == '-') {
        neg = *b == '-';
        b++;
    }
    if (b == e || e - b > 12) return false;
    int64_t v = 0;
    for (; b < e; b++) {
        if (*b < '0' || *b > '9') return false;
        v = v * 10 + (*b - '0');
    }
    *out = neg ? -v : v;
    return true;
}

// A decimal real field: optional sign, digits with at most one point, an
// optional exponent.  The value is the correctly rounded double: the digits
// are an exact integer (at most 17 significant digits here) scaled by an
// exact power of ten in one division or multiplication, which is correctly
// rounded when both operands are exact (|exponent| <= 22).
bool parse_real(const char *b, const char *e, double empty, double *out) {
    trim(b, e);
    if (b == e) {
        *out = empty;
        return true;
    }
    bool neg = false;
    if (*b == '+' || *b == '-') {
        neg = *b == '-';
        b++;
    }
    uint64_t mant = 0;
    int digits = 0, frac = 0;
    bool point = false, any = false;
    for (; b < e && ((*b >= '0' && *b <= '9') || *b == '.'); b++) {
        if (*b == '.') {
            if (point) return false;
            point = true;
            continue;
        }
        any = true;
        if (digits == 0 && *b == '0') {
            if (point) frac++;
            continue;
        }
        if (++digits > 17) return false;
        mant = mant * 10 + (uint64_t)(*b - '0');
        if (point) frac++;
    }
    if (!any) return false;
    int ex = 0;
    if (b < e && (*b == 'e' || *b == 'E')) {
        b++;
        bool eneg = false;
        if (b < e && (*b == '+' || *b == '-')) {
            eneg = *b == '-';
            b++;
        }
        if (b == e) return false;
        int v = 0;
        for (; b < e; b++) {
            if (*b < '0' || *b > '9' || v > 1000) return false;
            v = v * 10 + (*b - '0');
        }
        ex = eneg ? -v : v;
    }
    if (b != e) return false;
    static const double P10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                   1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    if (mant > (1ull << 53)) return false;  // not exact as a double
    const int scale = ex - frac;
    double v = (double)mant;
    if (mant != 0) {
        if (scale < -22 || scale > 22) return false;
        v = scale < 0 ? v / P10[-scale] : v * P10[scale];
    }
    *out = neg ? -v : v;
    return true;
}

// encode_token of the reference's Cython layer: bytes [b, b + n) of the
// padded line, spaces and NULs as '_'.
inline void token(const char *line, int from, int n, uint8_t *dst) {
    for (int i = 0; i < n; i++) {
        const char c = line[from + i];
        dst[i] = (c == ' ' || c == 0) ? '_' : (uint8_t)c;
    }
}

template <typename T>
inline void put(uint8_t *row, int off, T v) {
    std::memcpy(row + off, &v, sizeof v);
}

// One ATOM/HETATM line (without its terminator, `len` bytes) padded to 80
// columns with spaces; false when a field is not in a plain form.
bool parse_atom(const char *text, int64_t len, uint8_t *row) {
    char line[81];
    const int n = len < 80 ? (int)len : 80;
    std::memcpy(line, text, (size_t)n);
    std::memset(line + n, ' ', (size_t)(80 - n));
    line[80] = 0;
    for (int i = 0; i < 80; i++)
        if ((unsigned char)line[i] < 0x20 || (unsigned char)line[i] > 0x7e) return false;
    int64_t serial = 0, resseq = 0;
    double x[3], occ = 0.0, temp = 0.0;
    if (!parse_int(line + 6, line + 11, 0, &serial) || serial < INT32_MIN || serial > INT32_MAX) return false;
    if (!parse_int(line + 22, line + 26, 0, &resseq)) return false;
    for (int d = 0; d < 3; d++) {
        const char *b = line + 30 + 8 * d, *e = b + 8;
        const char *tb = b, *te = e;
        trim(tb, te);
        if (tb == te) return false;  // an empty coordinate is an error of the general reader
        if (!parse_real(b, e, 0.0, &x[d])) return false;
    }
    if (!parse_real(line + 54, line + 60, 0.0, &occ) || !parse_real(line + 60, line + 66, 0.0, &temp)) return false;
    // charge (columns 79-80): "n+", "n-", a signed integer, or blank
    int64_t charge = 0;
    {
        const char *b = line + 78, *e = line + 80;
        trim(b, e);
        if (b < e) {
            const char last = e[-1];
            if ((last == '+' || last == '-') && e - b >= 2) {
                bool digits = true;
                for (const char *p = b; p < e - 1; p++) digits = digits && *p >= '0' && *p <= '9';
                if (!digits) return false;
                parse_int(b, e - 1, 0, &charge);
                if (last == '-') charge = -charge;
            } else if (!parse_int(b, e, 0, &charge)) {
                return false;
            }
            if (charge < -128 || charge > 127) return false;
        }
    }
    std::memset(row, 0, ROW);
    put(row, O_X, x[0]);
    put(row, O_X + 8, x[1]);
    put(row, O_X + 16, x[2]);
    put(row, O_OCC, (float)occ);
    put(row, O_TEMP, (float)temp);
    put(row, O_SERIAL, (int32_t)serial);
    token(line, 12, 4, row + O_NAME);
    row[O_ALT] = (uint8_t)line[16];
    token(line, 17, 3, row + O_RES);
    row[O_RES + 3] = 0;
    row[O_CHAIN] = (uint8_t)line[20];
    row[O_CHAIN + 1] = (uint8_t)line[21];
    if (resseq < INT32_MIN || resseq > INT32_MAX) return false;
    put(row, O_RESSEQ, (int32_t)resseq);
    row[O_ICODE] = (uint8_t)line[26];
    token(line, 72, 4, row + O_SEG);
    token(line, 76, 2, row + O_ELEM);
    put(row, O_CHARGE, (int8_t)charge);
    return true;
}

inline bool starts(const char *p, int64_t n, const char *lit) {
    const int64_t k = (int64_t)std::strlen(lit);
    return n >= k && std::memcmp(p, lit, (size_t)k) == 0;
}

}  // namespace

extern "C" pjg_status pjg_parse_pdb(const char *text, int64_t len, int32_t flags, void *records, int64_t capacity,
                                    int64_t *n_atoms, int64_t *end_offset, int64_t *stop_offset) {
    if (!text || len < 0 || !n_atoms || !end_offset || !stop_offset || (capacity > 0 && !records))
        return PJG_ERR_INVALID;
    uint8_t *out = static_cast<uint8_t *>(records);
    int64_t count = 0;
    *end_offset = len;
    *stop_offset = -1;
    int64_t pos = 0;
    auto stop = [&](int64_t at) {
        *stop_offset = at;
        *end_offset = at;
        *n_atoms = count;
        return PJG_ERR_INVALID;
    };
    while (pos < len) {
        const char *line = text + pos;
        const char *nl = static_cast<const char *>(std::memchr(line, '\n', (size_t)(len - pos)));
        const int64_t full = nl ? (nl - line) + 1 : len - pos;  // with its terminator
        int64_t body = nl ? full - 1 : full;
        if (body > 0 && line[body - 1] == '\r') body--;
        // a carriage return inside a line ends a line for a text-mode
        // reader: leave such files to the general reader
        if (std::memchr(line, '\r', (size_t)body)) return stop(pos);
        const bool atom = starts(line, body, "ATOM");
        const bool het = starts(line, body, "HETATM") && !(flags & PJG_PDB_SKIP_HETATM);
        if (atom || het) {
            // the general reader rejects a record shorter than 54 characters
            // counted with a one-character line terminator
            if (body + (nl ? 1 : 0) < 54 || count >= capacity || !parse_atom(line, body, out + ROW * count))
                return stop(pos);
            count++;
        } else if (starts(line, body, "ENDMDL")) {
            if (!(flags & PJG_PDB_IGNORE_ENDMDL)) {
                *end_offset = pos;
                break;
            }
        } else if (body >= 5) {
            char low[5];
            for (int i = 0; i < 5; i++) low[i] = (char)(line[i] >= 'A' && line[i] <= 'Z' ? line[i] + 32 : line[i]);
            if (std::memcmp(low, "data_", 5) == 0 || std::memcmp(low, "loop_", 5) == 0) return stop(pos);
        }
        pos += full;
    }
    *n_atoms = count;
    return PJG_OK;
}
