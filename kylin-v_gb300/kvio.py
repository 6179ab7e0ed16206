"""Binary file formats of the Holstein TDVP path.

* ``.mps``  -- reference format, holstein/state.h:107-157: int32 tag 111, int32 ns,
  then per site int32 nblocks and per block int32 shape[3], int32 qn[3] and the
  complex128 row-major data; a trailing newline byte.
* ``.mpo``  -- the same with rank 4 and tag 112 (holstein/operator.h:94-143).
* ``.kvt``  -- one block-sparse tensor of any rank (used for golden vectors):
  int32 magic "KVT1", int32 rank, int32 dirs[rank], int32 nblocks, then per block
  int32 shape[rank], int32 qn[rank], complex128 data.

A tensor is held on the host as :class:`BlockTensor`: the leg directions and an
ordered list of ``(qn tuple, ndarray)`` blocks, the ndarray's shape being the
block shape (the reference's ``Block<Rank>``, holstein/block.h:23-166).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

MPS_TAG = 111
MPO_TAG = 112
KVT_MAGIC = 0x3154564B


@dataclass
class BlockTensor:
    dirs: tuple
    blocks: list = field(default_factory=list)  # [(qn tuple, complex128 ndarray)]

    @property
    def rank(self) -> int:
        return len(self.dirs)

    def copy(self) -> "BlockTensor":
        return BlockTensor(tuple(self.dirs), [(q, a.copy()) for q, a in self.blocks])

    def as_dict(self) -> dict:
        """Blocks keyed by (qn, shape); equal keys are summed (the reference's
        push_back_ch merge rule, holstein/tensor.h:172-185)."""
        out: dict = {}
        for q, a in self.blocks:
            k = (tuple(q), tuple(a.shape))
            out[k] = out[k] + a if k in out else a.copy()
        return out

    def norm(self) -> float:
        return float(np.sqrt(sum(np.vdot(a, a).real for _, a in self.blocks)))

    def legs(self) -> list:
        """Per leg the map charge -> dimension (the reference's leg_ maps)."""
        out = [dict() for _ in self.dirs]
        for q, a in self.blocks:
            for i, (c, d) in enumerate(zip(q, a.shape)):
                out[i][c] = d
        return out


def _read_blocks(buf: bytes, off: int, rank: int, nb: int):
    blocks = []
    for _ in range(nb):
        sh = struct.unpack_from(f"<{rank}i", buf, off)
        off += 4 * rank
        qn = struct.unpack_from(f"<{rank}i", buf, off)
        off += 4 * rank
        n = int(np.prod(sh))
        a = np.frombuffer(buf, dtype="<c16", count=n, offset=off).reshape(sh).copy()
        off += 16 * n
        blocks.append((tuple(qn), a))
    return blocks, off


def _write_blocks(f, blocks, rank):
    for qn, a in blocks:
        a = np.ascontiguousarray(a, dtype="<c16")
        assert a.ndim == rank
        f.write(struct.pack(f"<{rank}i", *a.shape))
        f.write(struct.pack(f"<{rank}i", *qn))
        f.write(a.tobytes())


def read_train(path: str, rank: int) -> list:
    """Read a .mps (rank 3) or .mpo (rank 4) file into a list of BlockTensors."""
    with open(path, "rb") as f:
        buf = f.read()
    tag, ns = struct.unpack_from("<2i", buf, 0)
    want = MPS_TAG if rank == 3 else MPO_TAG
    if tag != want:
        raise ValueError(f"{path}: tag {tag}, expected {want}")
    dirs = (1, 1, -1) if rank == 3 else (1, 1, -1, -1)
    off = 8
    sites = []
    for _ in range(ns):
        (nb,) = struct.unpack_from("<i", buf, off)
        off += 4
        blocks, off = _read_blocks(buf, off, rank, nb)
        sites.append(BlockTensor(dirs, blocks))
    return sites


def write_train(path: str, sites: list, rank: int) -> None:
    tag = MPS_TAG if rank == 3 else MPO_TAG
    with open(path, "wb") as f:
        f.write(struct.pack("<2i", tag, len(sites)))
        for t in sites:
            f.write(struct.pack("<i", len(t.blocks)))
            _write_blocks(f, t.blocks, rank)
        f.write(b"\n")


def read_mps(path: str) -> list:
    return read_train(path, 3)


def read_mpo(path: str) -> list:
    return read_train(path, 4)


def write_mps(path: str, sites: list) -> None:
    write_train(path, sites, 3)


def write_mpo(path: str, sites: list) -> None:
    write_train(path, sites, 4)


def read_kvt(path: str) -> BlockTensor:
    with open(path, "rb") as f:
        buf = f.read()
    magic, rank = struct.unpack_from("<2i", buf, 0)
    if magic != KVT_MAGIC:
        raise ValueError(f"{path}: not a KVT file")
    dirs = struct.unpack_from(f"<{rank}i", buf, 8)
    off = 8 + 4 * rank
    (nb,) = struct.unpack_from("<i", buf, off)
    blocks, _ = _read_blocks(buf, off + 4, rank, nb)
    return BlockTensor(tuple(dirs), blocks)


def write_kvt(path: str, t: BlockTensor) -> None:
    with open(path, "wb") as f:
        f.write(struct.pack("<2i", KVT_MAGIC, t.rank))
        f.write(struct.pack(f"<{t.rank}i", *t.dirs))
        f.write(struct.pack("<i", len(t.blocks)))
        _write_blocks(f, t.blocks, t.rank)
