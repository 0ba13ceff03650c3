// Host reader of the reference's FastASCII particle files (one particle per
// line, the fields of the set's "fields" list in order, vector components
// as separate numbers).
//
// Line rules (InputOutput/ASCII.cpp:374-403, formatLine): everything from
// '#' on is a comment; the line is trimmed; each of " ;()[]{}\t" is a
// separator (turned into ','), runs of separators count once, leading and
// trailing separators are dropped; empty lines are skipped.  A particle line
// must hold exactly the declared number of numbers (ASCII.cpp:165-173).
// Numbers (InputOutput/FastASCII.cpp:47-117, readField): each column is
// parsed from the start of the remaining text as its type's std::sto*
// function would -- float as strtof, int as strtol into int range, unsigned
// as strtoul -- then the text continues after the next separator; a column
// with no number, or one out of range, is an error.
#include <cerrno>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "aqua_gb300.h"

namespace {

bool
is_space(char c)
{
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' ||
           c == '\r';
}

bool
is_separator(char c)
{
    return c == ' ' || c == ';' || c == '(' || c == ')' || c == '[' ||
           c == ']' || c == '{' || c == '}' || c == '\t';
}

// formatLine of [b, e) into `out` (fields joined by single commas)
void
format_line(const char* b, const char* e, std::string& out)
{
    out.clear();
    const char* hash = static_cast<const char*>(std::memchr(b, '#', e - b));
    if (hash)
        e = hash;
    while (b < e && is_space(*b))
        b++;
    while (e > b && is_space(e[-1]))
        e--;
    bool pending = false;  // a separator seen since the last kept character
    for (const char* p = b; p < e; p++) {
        const char c = *p;
        if (c == ',' || is_separator(c)) {
            pending = true;
            continue;
        }
        if (pending && !out.empty())
            out.push_back(',');
        pending = false;
        out.push_back(c);
    }
}

uint32_t
count_fields(const std::string& l)
{
    if (l.empty())
        return 0;
    uint32_t n = 1;
    for (char c : l)
        n += (c == ',');
    return n;
}

// parses one column at `p` (NUL-terminated); returns false on error
bool
parse_column(const char*& p, int32_t type, uint32_t* dst)
{
    char* end = nullptr;
    errno = 0;
    if (type == AQUA_COLUMN_FLOAT) {
        const float v = std::strtof(p, &end);
        if (end == p || errno == ERANGE)
            return false;
        std::memcpy(dst, &v, 4);
    } else if (type == AQUA_COLUMN_INT) {
        const long v = std::strtol(p, &end, 10);
        if (end == p || errno == ERANGE || v < INT_MIN || v > INT_MAX)
            return false;
        const int32_t w = (int32_t)v;
        std::memcpy(dst, &w, 4);
    } else {
        const unsigned long v = std::strtoul(p, &end, 10);
        if (end == p || errno == ERANGE)
            return false;
        const uint32_t w = (uint32_t)v;
        std::memcpy(dst, &w, 4);
    }
    p = end;
    const char* comma = std::strchr(p, ',');
    if (comma)
        p = comma + 1;
    return true;
}

} // namespace

extern "C" aqua_status
aqua_read_fastascii(const char* path, uint32_t n_cols, const int32_t* col_types,
                    void* out, uint64_t max_rows, uint64_t* n_rows,
                    uint64_t* bad_line)
{
    if (!path || !n_rows)
        return AQUA_ERR_INVALID;
    if (out && (n_cols == 0 || !col_types))
        return AQUA_ERR_INVALID;
    for (uint32_t j = 0; out && j < n_cols; j++)
        if (col_types[j] < AQUA_COLUMN_FLOAT || col_types[j] > AQUA_COLUMN_UINT)
            return AQUA_ERR_INVALID;
    *n_rows = 0;
    if (bad_line)
        *bad_line = 0;
    FILE* f = std::fopen(path, "rb");
    if (!f)
        return AQUA_ERR_IO;
    std::vector<char> text;
    char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0)
        text.insert(text.end(), chunk, chunk + got);
    const bool read_error = std::ferror(f) != 0;
    std::fclose(f);
    if (read_error)
        return AQUA_ERR_IO;

    uint32_t* words = static_cast<uint32_t*>(out);
    std::string line;
    uint64_t rows = 0, line_no = 0;
    const char* p = text.data();
    const char* end = p + text.size();
    while (p < end) {
        const char* nl = static_cast<const char*>(std::memchr(p, '\n', end - p));
        const char* e = nl ? nl : end;
        line_no++;
        format_line(p, e, line);
        p = nl ? nl + 1 : end;
        if (line.empty())
            continue;
        if (!out) {
            rows++;
            continue;
        }
        if (count_fields(line) != n_cols) {
            if (bad_line)
                *bad_line = line_no;
            *n_rows = rows;
            return AQUA_ERR_FORMAT;
        }
        if (rows >= max_rows) {
            *n_rows = rows;
            return AQUA_ERR_CAPACITY;
        }
        const char* q = line.c_str();
        uint32_t* row = words + rows * (uint64_t)n_cols;
        for (uint32_t j = 0; j < n_cols; j++)
            if (!parse_column(q, col_types[j], row + j)) {
                if (bad_line)
                    *bad_line = line_no;
                *n_rows = rows;
                return AQUA_ERR_FORMAT;
            }
        rows++;
    }
    *n_rows = rows;
    return AQUA_OK;
}
