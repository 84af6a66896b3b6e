"""The reference's on-disk MPS format (restart / interchange), host side.

block2 keeps an MPS as files in its scratch directory:

* ``F.MPS.<tag>.-1`` -- MPS::save_data_to (src/dmrg/mps.hpp:2505-2514):
  int32 n_sites, int32 center, int32 dot, n_sites canonical-form characters,
  n_sites uint8 "tensor present" flags;
* ``F.MPS.<tag>.<i>`` -- one site tensor, SparseMatrix::save_data with its
  info (src/core/sparse_matrix.hpp:555-571, 954-975): the SparseMatrixInfo
  (uint64 delta quantum, int32 n blocks, uint64 labels[n], uint16 bra
  states[n], uint16 ket states[n], uint32 block shifts[n], uint8 fermion
  flag, uint8 wavefunction / shift-size flags) then the matrix (float64
  factor, uint64 total_memory, float64 data[total_memory]);
* ``F.MPS.INFO.<tag>.LEFT.<i>`` / ``.RIGHT.<i>`` -- the bond StateInfos,
  StateInfo::save_data (src/core/state_info.hpp:101-105): int32 total states,
  int32 n, uint64 labels[n], uint16 counts[n] padded to 4 bytes.

The layouts assume the reference's default build (16-bit ``ubond_t``, no
compressed tensor storage); other builds are rejected when read.  Readers
return numpy arrays; ``SiteTensor.block(i)`` views block i, and ``data`` can
go to the GPU as the flat wavefunction the effective-Hamiltonian kernels read
(the same block order and shifts).  Writers reproduce the files byte for byte.
"""
from __future__ import annotations

import os
import struct
from dataclasses import dataclass, field

import numpy as np


@dataclass
class StateInfoData:
    n_states_total: int
    quanta: np.ndarray          # uint64[n]
    n_states: np.ndarray        # uint16[n]
    pad: bytes = b""            # the padding half-word of an odd n, kept as read

    def to_bytes(self) -> bytes:
        n = self.quanta.size
        body = struct.pack("<ii", self.n_states_total, n) + self.quanta.astype("<u8").tobytes()
        body += self.n_states.astype("<u2").tobytes()
        if n & 1:
            body += self.pad if len(self.pad) == 2 else b"\0\0"
        return body


@dataclass
class SiteTensor:
    delta_quantum: int
    quanta: np.ndarray          # uint64[n] block labels
    n_bra: np.ndarray           # uint16[n] rows of each block
    n_ket: np.ndarray           # uint16[n] columns of each block
    shifts: np.ndarray          # uint32[n] block offsets into data
    is_fermion: int
    flags: int                  # bit 0: wavefunction; bits 2..: block-shift size code
    factor: float
    data: np.ndarray            # float64[total_memory]

    @property
    def is_wavefunction(self) -> bool:
        return bool(self.flags & 1)

    def block(self, i: int) -> np.ndarray:
        r, c, s = int(self.n_bra[i]), int(self.n_ket[i]), int(self.shifts[i])
        return self.data[s:s + r * c].reshape(r, c)

    def to_bytes(self) -> bytes:
        n = self.quanta.size
        b = struct.pack("<Qi", self.delta_quantum, n)
        b += self.quanta.astype("<u8").tobytes() + self.n_bra.astype("<u2").tobytes()
        b += self.n_ket.astype("<u2").tobytes() + self.shifts.astype("<u4").tobytes()
        b += struct.pack("<BB", self.is_fermion, self.flags)
        b += struct.pack("<dQ", self.factor, self.data.size) + self.data.astype("<f8").tobytes()
        return b


@dataclass
class MPSHeader:
    n_sites: int
    center: int
    dot: int
    canonical_form: str
    present: np.ndarray         # uint8[n_sites]

    def to_bytes(self) -> bytes:
        return (struct.pack("<iii", self.n_sites, self.center, self.dot) +
                self.canonical_form.encode("ascii") + self.present.astype(np.uint8).tobytes())


@dataclass
class MPSFiles:
    header: MPSHeader
    tensors: list = field(default_factory=list)       # SiteTensor or None per site
    left_dims: list = field(default_factory=list)     # StateInfoData per bond (0..n_sites)
    right_dims: list = field(default_factory=list)


class FormatError(ValueError):
    pass


def _take(buf: bytes, pos: int, n: int) -> tuple[bytes, int]:
    if pos + n > len(buf):
        raise FormatError("file ends early")
    return buf[pos:pos + n], pos + n


def parse_state_info(buf: bytes) -> StateInfoData:
    (tot, n), pos = struct.unpack("<ii", buf[:8]), 8
    if n < 0:
        raise FormatError("negative label count")
    q, pos = _take(buf, pos, 8 * n)
    c, pos = _take(buf, pos, 2 * n)
    pad = b""
    if n & 1:
        pad, pos = _take(buf, pos, 2)
    if pos != len(buf):
        raise FormatError("trailing bytes after a StateInfo (not a 16-bit ubond_t build?)")
    return StateInfoData(tot, np.frombuffer(q, "<u8").copy(), np.frombuffer(c, "<u2").copy(), pad)


def parse_site_tensor(buf: bytes) -> SiteTensor:
    dq, n = struct.unpack("<Qi", buf[:12])
    pos = 12
    if n < 0:
        raise FormatError("negative block count")
    q, pos = _take(buf, pos, 8 * n)
    rb, pos = _take(buf, pos, 2 * n)
    ck, pos = _take(buf, pos, 2 * n)
    sh, pos = _take(buf, pos, 4 * n)
    ff, pos = _take(buf, pos, 2)
    fac_tm, pos = _take(buf, pos, 16)
    factor, total = struct.unpack("<dQ", fac_tm)
    if total == 0xFFFFFFFFFFFFFFFF:
        raise FormatError("compressed tensor storage is not supported")
    d, pos = _take(buf, pos, 8 * total)
    if pos != len(buf):
        raise FormatError("trailing bytes after a site tensor (not a 16-bit ubond_t build?)")
    t = SiteTensor(dq, np.frombuffer(q, "<u8").copy(), np.frombuffer(rb, "<u2").copy(),
                   np.frombuffer(ck, "<u2").copy(), np.frombuffer(sh, "<u4").copy(), ff[0], ff[1],
                   factor, np.frombuffer(d, "<f8").copy())
    # the blocks tile data exactly (initialize_block_shifts, sparse_matrix.hpp:617-630)
    sizes = t.n_bra.astype(np.int64) * t.n_ket.astype(np.int64)
    if n and (np.any(t.shifts.astype(np.int64) != np.concatenate([[0], np.cumsum(sizes)[:-1]]))
              or int(sizes.sum()) != total):
        raise FormatError("block shifts do not tile the tensor data")
    return t


def parse_header(buf: bytes) -> MPSHeader:
    ns, center, dot = struct.unpack("<iii", buf[:12])
    if ns <= 0 or len(buf) != 12 + 2 * ns:
        raise FormatError("MPS header size does not match its site count")
    form = buf[12:12 + ns].decode("ascii")
    return MPSHeader(ns, center, dot, form, np.frombuffer(buf[12 + ns:], np.uint8).copy())


def _read(path: str) -> bytes:
    with open(path, "rb") as f:
        return f.read()


def _write(path: str, data: bytes):
    with open(path, "wb") as f:
        f.write(data)


def load_mps(scratch: str, tag: str = "KET") -> MPSFiles:
    """Every file of MPS `tag` in a reference scratch directory."""
    h = parse_header(_read(os.path.join(scratch, f"F.MPS.{tag}.-1")))
    m = MPSFiles(h)
    for i in range(h.n_sites):
        p = os.path.join(scratch, f"F.MPS.{tag}.{i}")
        m.tensors.append(parse_site_tensor(_read(p)) if h.present[i] and os.path.exists(p) else None)
    for side, lst in (("LEFT", m.left_dims), ("RIGHT", m.right_dims)):
        i = 0
        while os.path.exists(os.path.join(scratch, f"F.MPS.INFO.{tag}.{side}.{i}")):
            lst.append(parse_state_info(_read(os.path.join(scratch, f"F.MPS.INFO.{tag}.{side}.{i}"))))
            i += 1
    return m


def save_mps(scratch: str, m: MPSFiles, tag: str = "KET"):
    """Write MPS `tag` in the reference's layout (the reference can load it)."""
    os.makedirs(scratch, exist_ok=True)
    _write(os.path.join(scratch, f"F.MPS.{tag}.-1"), m.header.to_bytes())
    for i, t in enumerate(m.tensors):
        if t is not None:
            _write(os.path.join(scratch, f"F.MPS.{tag}.{i}"), t.to_bytes())
    for side, lst in (("LEFT", m.left_dims), ("RIGHT", m.right_dims)):
        for i, s in enumerate(lst):
            _write(os.path.join(scratch, f"F.MPS.INFO.{tag}.{side}.{i}"), s.to_bytes())
