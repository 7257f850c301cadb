/* ORACLE -- test infrastructure, never the product.
 *
 * A restatement, in plain C, of the reference's text Loader: Loader::Host
 * (core/operator.cpp:24-48) walking a bulk's bytes, and
 * GetValueOfItemBySwitch (com/cpp/com.cu:33-44) converting one item.
 *
 *   - Bytes accumulate into the current item.  A column delimiter ends the
 *     item, which is converted into column `col` of row `row`; col advances.
 *   - A row delimiter starts the next row (col = 0) and discards whatever
 *     item text is pending: a line's last field is stored only when a column
 *     delimiter follows it, as in SSB's "a|b|c|\n" lines.
 *   - The row count is the number of row delimiters (a last line without
 *     one is not counted).
 *   - Int32 items convert as atoi, Int64 items as atol: (int)strtol /
 *     strtol(s, NULL, 10) on LP64.  The conversion here is written out
 *     (leading isspace, optional sign, decimal digits, clamp to the long
 *     range on overflow, Int32 keeps the low 32 bits) and is checked against
 *     the C library's own atoi/atol by tests/test_loader.py.
 *
 * Where the reference's behaviour is undefined the restatement, and the
 * GPU loader, choose: fields past the schema's last column are ignored
 * (the reference writes past its column buffers); columns a row does not
 * reach are zero; the fields of a last line without a row delimiter are not
 * stored (the reference writes them past its row count); an item longer than
 * 4095 bytes (it would overflow the reference's item buffer,
 * operator.cpp:25) is an error, reported as -1.
 */
#include <stddef.h>
#include <stdint.h>
#include <string.h>

static int is_space(unsigned char c) { return c == ' ' || (c >= '\t' && c <= '\r'); }

/* strtol(s, NULL, 10) over bytes [s, e) followed by a NUL (LP64 long). */
static long long parse_long(const unsigned char* s, const unsigned char* e) {
  while (s < e && is_space(*s)) s++;
  int neg = 0;
  if (s < e && (*s == '+' || *s == '-')) {
    neg = *s == '-';
    s++;
  }
  unsigned long long acc = 0;
  const unsigned long long lim = neg ? 9223372036854775808ull : 9223372036854775807ull;
  int over = 0;
  for (; s < e && *s >= '0' && *s <= '9'; s++) {
    unsigned d = (unsigned)(*s - '0');
    if (over) continue;
    if (acc > (lim - d) / 10) {
      over = 1;
      continue;
    }
    acc = acc * 10 + d;
  }
  if (over) return neg ? (long long)(-9223372036854775807ll - 1) : 9223372036854775807ll;
  return neg ? (long long)(0ull - acc) : (long long)acc;
}

/* Loads `text` into ncols columns of int32 (types[c] == 2) or int64
 * (types[c] == 3, ValType numbering of com/svm.proto:62-72).  out[c] points
 * to cap_rows values (fields of rows >= cap_rows are not stored).  Returns
 * the row count, or -1 for an item longer than 4095 bytes. */
long long svm_oracle_load_text(const char* text, unsigned long long bytes, char col_delim, char row_delim, int ncols,
                               const int* types, void* const* out, unsigned long long cap_rows) {
  const unsigned char* p = (const unsigned char*)text;
  unsigned long long row = 0;
  int col = 0;
  unsigned long long start = 0; /* first byte of the pending item */
  for (int c = 0; c < ncols; c++) memset(out[c], 0, cap_rows * (types[c] == 3 ? 8 : 4));
  for (unsigned long long i = 0; i < bytes; i++) {
    const char ch = (char)p[i];
    if (ch == col_delim) {
      if (i - start > 4095) return -1;
      if (col < ncols && row < cap_rows) {
        const long long v = parse_long(p + start, p + i);
        if (types[col] == 3)
          ((long long*)out[col])[row] = v;
        else
          ((int32_t*)out[col])[row] = (int32_t)(uint32_t)(unsigned long long)v;
      }
      col++;
      start = i + 1;
    } else if (ch == row_delim) {
      col = 0;
      row++;
      start = i + 1;
    }
  }
  return (long long)row;
}
