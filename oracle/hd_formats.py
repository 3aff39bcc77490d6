"""Test infrastructure only (the oracle): a plain-Python restatement of the
reference's result-file formats, used to check the device implementations.
Nothing in the product imports this file.

- dump (include/hamming/hamming.hh:63-73): the full n x n matrix, entries
  `(*this)[{i, j}]` (0 on the diagonal, symmetric), ", " between entries,
  one line per row.
- from_lower_triangular<T> (hamming.hh:152-166): every line is split on ','
  by std::getline while the stream is good, so each line yields all of its
  comma-separated fields (an empty line or a trailing comma yields an empty
  field); each field goes through std::stoi and safe_int_cast<T>
  (include/hamming/hamming_impl.hh:37-45: above max saturates, below 0 wraps);
  nsamples = (round(sqrt(8 * size + 1)) + 1) / 2 (hamming.hh:18-20, 57-61).
- from_csv (hamming.hh:34-55, src/hamming.cc:23-25): nsamples = number of
  '\\n'; result has nsamples(nsamples+1)/2 entries (zero-filled); line i
  (0-based, including a last line without '\\n') contributes its first i
  fields to result[i(i-1)/2 + j]; once the line's stream is exhausted,
  std::getline leaves the previous field in place, so missing fields repeat
  the line's last field; values are std::stoi truncated to uint8.
- std::stoi: leading C-locale whitespace, an optional sign, then at least one
  decimal digit (anything after the digits is ignored); no digits raises
  std::invalid_argument ("stoi"; ValueError through pybind11), a value
  outside int raises std::out_of_range ("stoi"; IndexError).
"""
from __future__ import annotations

import math

import numpy as np

_WS = b" \t\n\v\f\r"
INT_MAX, INT_MIN = 2**31 - 1, -(2**31)


def stoi(field: bytes) -> int:
    k = 0
    while k < len(field) and field[k] in _WS:
        k += 1
    sign = 1
    if k < len(field) and field[k] in b"+-":
        sign = -1 if field[k] == ord("-") else 1
        k += 1
    start = k
    while k < len(field) and 48 <= field[k] <= 57:
        k += 1
    if k == start:
        raise ValueError("stoi")
    v = sign * int(field[start:k])
    if v > INT_MAX or v < INT_MIN:
        raise IndexError("stoi")
    return v


def safe_int_cast(v: int, dtype) -> int:
    mx = np.iinfo(dtype).max
    return mx if v > mx else v % (mx + 1)


def lines_of(data: bytes) -> list[bytes]:
    """std::getline over the whole file: a final '\\n' ends the last line."""
    if not data:
        return []
    parts = data.split(b"\n")
    if data.endswith(b"\n"):
        parts = parts[:-1]
    return parts


def nsamples_of(entries: int) -> int:
    return (int(round(math.sqrt(8 * entries + 1))) + 1) // 2


def from_lower_triangular(data: bytes, dtype=np.uint8):
    out = []
    for line in lines_of(data):
        for field in line.split(b","):
            out.append(safe_int_cast(stoi(field), dtype))
    lt = np.array(out, dtype=dtype)
    return lt, nsamples_of(lt.size)


def from_csv(data: bytes):
    n = data.count(b"\n")
    lt = np.zeros(n * (n + 1) // 2, dtype=np.uint8)
    for i, line in enumerate(lines_of(data)):
        fields = line.split(b",")
        for j in range(i):
            v = stoi(fields[min(j, len(fields) - 1)])
            lt[i * (i - 1) // 2 + j] = v % 256
    return lt, n


def entry(lt, i: int, j: int) -> int:
    if i == j:
        return 0
    if i < j:
        i, j = j, i
    return int(lt[i * (i - 1) // 2 + j])


def dump_text(lt, n: int) -> bytes:
    rows = []
    for i in range(n):
        rows.append(", ".join(str(entry(lt, i, j)) for j in range(n)).encode() + b"\n")
    return b"".join(rows)
