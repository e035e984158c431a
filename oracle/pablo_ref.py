"""CPU oracle for the bitstream hot path (test infrastructure only).

Nothing in the product imports this module: only ``tests/``, ``__graft_entry__.smoke()`` and
the ``cpu_baseline`` leg of ``bench.py`` use it, as the checker.

It restates, in plain Python/numpy, what the reference computes on its hot path:

* ``transpose_ref``: the byte -> basis-plane transpose.  Restates the reference's CPU path
  ``transpose_bytestream_to_bitstream_py`` (``bitgen/bitstream.py:228-258``): plane ``i`` holds
  bit ``7 - i`` of each byte (``np.unpackbits`` big-endian order), characters are packed 32 to a
  ``uint32`` word with character ``32w + j`` at bit ``31 - j`` (``bitstream.py:248-256``).  The
  reference's CUDA kernel produces the same layout (``bitgen/template/cuda/kernel.cu:60-100``).
* ``run_group``: a whole-stream interpreter of a Pablo program over Python big integers
  (bit ``p`` of an int = character position ``p``).  Semantics follow the reference's stream
  operators:

  - bitwise ops: ``bitgen/template/template.py:27-61``;
  - ``Advance(a, n)`` moves marks to higher positions and shifts zeros in at position 0
    (``template.py:63-70``; ``bitgen/bitstream.py:152-159``); ``Lookahead(a, n)`` is its mirror
    image (position p takes a[p + n], zeros enter past the end of the input);
  - ``MatchStar(M, C) = (((M & C) + C) ^ C) | M`` (``template.py:96-103``,
    ``bitgen/template/template_torch.py:392-407``);
  - ``ScanThru(M, C) = (M + C) & ~C`` (``template_torch.py:377-389``; the numpy template at
    ``template.py:88-94`` masks with ``~M``, which is a bug there);
  - additions are over the finite stream: the carry out of the last position is dropped
    (``template.py:80-85``);
  - ``while v`` repeats while any bit of ``v`` is set in the whole stream and ``if v`` tests the
    whole stream (``bitgen/inst/inst_block_while.py:137-153``, ``inst_block_if.py:314-342``);
  - ``SEL(c, a, b) = (c & a) | (~c & b)`` (``bitgen/inst/inst_sel.py:42-57``).

  The stream covers exactly ``n`` positions: bits at or beyond ``n`` do not exist, so they never
  make a ``while``/``if`` condition true and are never reported.
* ``count``: popcount of a result stream (``bitgen/bitstream.py:60-61``).
"""

from __future__ import annotations

import numpy as np

from bitgen_gb300.pablo import Group, If, Op, While


def transpose_ref(data) -> np.ndarray:
    """Bytes -> ``uint32[8, ceil(n/32)]`` basis planes in the reference layout."""
    a = np.frombuffer(bytes(data), dtype=np.uint8) if not isinstance(data, np.ndarray) else data.astype(np.uint8)
    n = a.size
    W = (n + 31) // 32
    pad = np.zeros(W * 32, dtype=np.uint8)
    pad[:n] = a
    bits = np.unpackbits(pad).reshape(W * 32, 8).T          # [8, n_pad]; row i = bit 7-i
    packed = np.packbits(bits, axis=-1, bitorder="big")      # [8, W*4] bytes, char 0 at MSB
    b = packed.reshape(8, W, 4).astype(np.uint32)
    return (b[..., 0] << 24) | (b[..., 1] << 16) | (b[..., 2] << 8) | b[..., 3]


def words_to_int(words: np.ndarray) -> int:
    """Reference-layout ``uint32`` words -> big int with bit p = position p."""
    w = np.asarray(words, dtype=np.uint32)
    if w.size == 0:
        return 0
    # bit (31-j) of word k is position 32k+j: reverse bits within each word, little-endian bytes
    b = w.astype(">u4").view(np.uint8)                      # big-endian bytes: char order within word
    bits = np.unpackbits(b)                                  # position order
    return int.from_bytes(np.packbits(bits, bitorder="little").tobytes(), "little")


def int_to_words(x: int, W: int) -> np.ndarray:
    """Big int (bit p = position p) -> reference-layout ``uint32[W]``."""
    nbytes = W * 4
    raw = np.frombuffer(x.to_bytes(nbytes, "little"), dtype=np.uint8)
    bits = np.unpackbits(raw, bitorder="little")             # position order
    return np.packbits(bits).view(">u4").astype(np.uint32)


def basis_ints(data) -> list:
    """The 8 basis streams as big ints (position order)."""
    a = np.frombuffer(bytes(data), dtype=np.uint8) if not isinstance(data, np.ndarray) else data.astype(np.uint8)
    out = []
    for i in range(8):
        bits = ((a >> (7 - i)) & 1).astype(np.uint8)
        out.append(int.from_bytes(np.packbits(bits, bitorder="little").tobytes(), "little"))
    return out


def advance(a: int, k: int, mask: int) -> int:
    return (a << k) & mask


def matchstar(m: int, c: int, mask: int) -> int:
    return ((((m & c) + c) & mask) ^ c) | m


def scanthru(m: int, c: int, mask: int) -> int:
    return ((m + c) & mask) & ~c & mask


def run_group(group: Group, data, n: int | None = None, max_iters: int = 1 << 24, want=None):
    """Run ``group`` over ``data`` (bytes) of length ``n``; return the result stream (int).

    With ``want`` (a list of variable names) return ``{name: value}`` for those variables
    after the program ran, in addition to the result: ``(result, values)``.
    """
    a = np.frombuffer(bytes(data), dtype=np.uint8) if not isinstance(data, np.ndarray) else data.astype(np.uint8)
    if n is None:
        n = a.size
    a = a[:n]
    mask = (1 << n) - 1
    env = {f"basis{i}": v for i, v in enumerate(basis_ints(a))}
    env["0"] = 0
    env["1"] = mask

    def ev(stmts):
        for s in stmts:
            if isinstance(s, Op):
                x = [env[v] for v in s.args]
                if s.op == "assign":
                    r = x[0]
                elif s.op == "not":
                    r = ~x[0] & mask
                elif s.op == "and":
                    r = x[0] & x[1]
                elif s.op == "or":
                    r = x[0] | x[1]
                elif s.op == "xor":
                    r = x[0] ^ x[1]
                elif s.op == "sel":
                    r = (x[0] & x[1]) | (~x[0] & x[2] & mask)
                elif s.op == "advance":
                    r = advance(x[0], s.shift, mask)
                elif s.op == "lookahead":
                    r = (x[0] & mask) >> s.shift
                elif s.op == "matchstar":
                    r = matchstar(x[0], x[1], mask)
                elif s.op == "scanthru":
                    r = scanthru(x[0], x[1], mask)
                else:
                    raise ValueError(s.op)
                env[s.dst] = r & mask
            elif isinstance(s, While):
                it = 0
                while env[s.cond] & mask:
                    ev(s.body)
                    it += 1
                    if it > max_iters:
                        raise RuntimeError("while loop did not terminate")
            elif isinstance(s, If):
                if env[s.cond] & mask:
                    ev(s.then)
                elif s.orelse is not None:
                    ev(s.orelse)

    ev(group.stmts)
    res = env[group.result] & mask
    if want is not None:
        return res, {k: env[k] & mask for k in want}
    return res


def count(x: int) -> int:
    return bin(x).count("1")
