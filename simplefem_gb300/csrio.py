"""Binary file formats shared by the tests, the golden fixtures and the bench.

``.csr``  : b"FEECCSR1", int64 [N, ncols, nnz, pdim], int32 A[N+1], int32 C[nnz],
            float64 V[nnz], float64 pos[N*pdim] (degree-of-freedom positions, optional).
``.vec``  : raw float64 array.
``.sol``  : int64 [N, K], float64 seconds, float64 x[N], float64 residual[N].
``.rb``   : int64 [N, num_colors], int32 F[N], int32 B[num_colors+1], int32 R[N].
``.coo``  : b"FEECCOO1", int64 [rows, cols, count], int32 row[count], int32 col[count],
            float64 value[count] (``SparseMatrix`` entries, sparse/sparsematrix.hpp:31-38).

The CSR arrays are exactly ``MatrixCSR``'s ``A``/``C``/``V`` (sparse/matcsr.hpp:117-119).
"""
from __future__ import annotations

import dataclasses
import gzip
import io
import os

import numpy as np

_MAGIC = b"FEECCSR1"


@dataclasses.dataclass
class CsrData:
    A: np.ndarray
    C: np.ndarray
    V: np.ndarray
    ncols: int
    pos: np.ndarray | None = None

    @property
    def n(self) -> int:
        return len(self.A) - 1

    @property
    def nnz(self) -> int:
        return len(self.C)


def _open(path, mode):
    return gzip.open(path, mode) if str(path).endswith(".gz") else open(path, mode)


def read_csr(path) -> CsrData:
    with _open(path, "rb") as f:
        buf = f.read()
    if buf[:8] != _MAGIC:
        raise ValueError(f"{path}: not a FEECCSR1 file")
    n, ncols, nnz, pdim = np.frombuffer(buf, np.int64, 4, 8)
    off = 40
    A = np.frombuffer(buf, np.int32, n + 1, off).copy(); off += 4 * (n + 1)
    C = np.frombuffer(buf, np.int32, nnz, off).copy(); off += 4 * nnz
    V = np.frombuffer(buf, np.float64, nnz, off).copy(); off += 8 * nnz
    pos = None
    if pdim:
        pos = np.frombuffer(buf, np.float64, n * pdim, off).copy().reshape(n, pdim)
    return CsrData(A, C, V, int(ncols), pos)


def write_csr(path, m: CsrData) -> None:
    pdim = 0 if m.pos is None else m.pos.shape[1]
    bio = io.BytesIO()
    bio.write(_MAGIC)
    bio.write(np.array([m.n, m.ncols, m.nnz, pdim], np.int64).tobytes())
    bio.write(np.ascontiguousarray(m.A, np.int32).tobytes())
    bio.write(np.ascontiguousarray(m.C, np.int32).tobytes())
    bio.write(np.ascontiguousarray(m.V, np.float64).tobytes())
    if pdim:
        bio.write(np.ascontiguousarray(m.pos, np.float64).tobytes())
    with _open(path, "wb") as f:
        f.write(bio.getvalue())


def read_vec(path, n=None) -> np.ndarray:
    with _open(path, "rb") as f:
        v = np.frombuffer(f.read(), np.float64).copy()
    if n is not None and len(v) != n:
        raise ValueError(f"{path}: expected {n} doubles, found {len(v)}")
    return v


def write_vec(path, v) -> None:
    with _open(path, "wb") as f:
        f.write(np.ascontiguousarray(v, np.float64).tobytes())


def read_sol(path):
    with _open(path, "rb") as f:
        buf = f.read()
    n, K = np.frombuffer(buf, np.int64, 2, 0)
    secs = float(np.frombuffer(buf, np.float64, 1, 16)[0])
    x = np.frombuffer(buf, np.float64, n, 24).copy()
    r = np.frombuffer(buf, np.float64, n, 24 + 8 * n).copy()
    return int(K), x, r, secs


def read_rainbow(path):
    with _open(path, "rb") as f:
        buf = f.read()
    n, nc = (int(v) for v in np.frombuffer(buf, np.int64, 2, 0))
    off = 16
    F = np.frombuffer(buf, np.int32, n, off).copy(); off += 4 * n
    B = np.frombuffer(buf, np.int32, nc + 1, off).copy(); off += 4 * (nc + 1)
    R = np.frombuffer(buf, np.int32, n, off).copy()
    return nc, F, B, R


def write_rainbow(path, nc, F, B, R) -> None:
    with _open(path, "wb") as f:
        f.write(np.array([len(F), nc], np.int64).tobytes())
        f.write(np.ascontiguousarray(F, np.int32).tobytes())
        f.write(np.ascontiguousarray(B, np.int32).tobytes())
        f.write(np.ascontiguousarray(R, np.int32).tobytes())


def exists(path) -> bool:
    return os.path.exists(path)


def write_coo(path, rows: int, cols: int, r, c, v) -> None:
    r = np.ascontiguousarray(r, np.int32); c = np.ascontiguousarray(c, np.int32); v = np.ascontiguousarray(v, np.float64)
    with _open(path, "wb") as f:
        f.write(b"FEECCOO1")
        f.write(np.array([rows, cols, len(r)], np.int64).tobytes())
        f.write(r.tobytes()); f.write(c.tobytes()); f.write(v.tobytes())


def read_coo(path):
    """(r, c, v, rows, cols) of a FEECCOO1 file."""
    with _open(path, "rb") as f:
        buf = f.read()
    if buf[:8] != b"FEECCOO1":
        raise ValueError(f"{path}: not a FEECCOO1 file")
    rows, cols, count = (int(x) for x in np.frombuffer(buf, np.int64, 3, 8))
    off = 32
    r = np.frombuffer(buf, np.int32, count, off).copy(); off += 4 * count
    c = np.frombuffer(buf, np.int32, count, off).copy(); off += 4 * count
    v = np.frombuffer(buf, np.float64, count, off).copy()
    return r, c, v, rows, cols
