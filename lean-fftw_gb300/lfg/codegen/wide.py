"""Lane-parallel schedules of the butterfly kernels (the lone-transform latency path).

On GB300 a binary64 warp instruction holds its SM sub-partition's FP64 pipe for 64 cycles
however few lanes are active, so a butterfly evaluated by one thread costs its operation
count times 64 cycles (208 for a twiddled radix 16).  The kernels' DAGs are shallow (depth 8
for that radix 16, at most 32 operations on one level), so a group of W lanes can evaluate
one butterfly level by level, one operation per lane per level: the serial cost becomes the
depth.

A schedule is a table the device kernel interprets.  Each lane group keeps a value table V
of binary64 values: V[0] = 1.0, V[1] = -0.0, then the kernel's constants, then its inputs,
then one slot per operation.  Every operation is issued as the fused multiply-add that the
straight-line codelet issues for it (`emit.kernel_body`, binary64 CUDA dialect):

    add(a, b)      fma(a, 1, b)          sub(a, b)      fma(-b, 1, a)
    mul(a, b)      fma(a, b, -0)         fma(a, b, c)   fma(a, b, c)
    fms(a, b, c)   fma(a, b, -c)         fnma(a, b, c)  fma(-a, b, c)

so the device computes the same operations on the same operands and every value keeps its
bits.  A level's descriptor for lane s names the slots of A, B and C, whether A and C are
negated (a sign flip, as the codelet's unary minus), and the slot the result goes to.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass
from typing import Dict, List, Tuple

from .kernel import butterfly_k
from .sexpr import cst_value

SLOT_BITS = 10
MAX_SLOTS = 1 << SLOT_BITS


@dataclass(frozen=True)
class WideSchedule:
    W: int                              # lanes per butterfly (power of two, <= 32)
    n_in: int
    consts: Tuple[int, ...]             # bit patterns of V[0 .. len(consts))
    levels: Tuple[Tuple[int, ...], ...]  # per level, W packed descriptors
    outs: Tuple[int, ...]               # V slots of the 2R outputs (re, im interleaved),
                                        # bit 15: the output is the slot's negation
    n_slots: int                        # the last one is the idle lanes' scratch slot

    @property
    def depth(self) -> int:
        return len(self.levels)

    @property
    def in_base(self) -> int:
        return len(self.consts)


def _bits(v: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", v))[0]


def pack_desc(a: int, b: int, c: int, neg_a: bool, neg_c: bool, out: int) -> int:
    """Descriptor of one lane's operation: A, B, C slots (10 bits each), negate A (bit 30),
    negate C (bit 31), result slot (bits 32-41), active (bit 42)."""
    for s in (a, b, c, out):
        assert 0 <= s < MAX_SLOTS
    return a | (b << 10) | (c << 20) | (int(neg_a) << 30) | (int(neg_c) << 31) | (out << 32) | (1 << 42)


def unpack_desc(d: int):
    if not (d >> 42) & 1:
        return None
    m = MAX_SLOTS - 1
    return (d & m, (d >> 10) & m, (d >> 20) & m, bool((d >> 30) & 1), bool((d >> 31) & 1),
            (d >> 32) & m)


def wide_schedule(fwd: bool, R: int, twiddled: bool) -> WideSchedule:
    k = butterfly_k(fwd, R, twiddled)
    consts: List[int] = [_bits(1.0), _bits(-0.0)]
    cslot: Dict[int, int] = {}
    # every DAG node is a value slot and a sign: a negation is exact (a sign flip), so it is
    # folded into the operands that read it instead of taking a level of its own
    slot_of: Dict[int, Tuple[int, bool]] = {}
    for i, op in enumerate(k.ops):                      # constants first
        if op[0] in ("cst", "zero"):
            b = _bits(cst_value(op[1]) if op[0] == "cst" else 0.0)
            if b not in cslot:
                cslot[b] = len(consts)
                consts.append(b)
            slot_of[k.n_in + i] = (cslot[b], False)
    in_base = len(consts)
    for i in range(k.n_in):
        slot_of[i] = (in_base + i, False)
    nxt = in_base + k.n_in
    depth: Dict[int, int] = {i: 0 for i in range(k.n_in)}
    per_level: Dict[int, List[int]] = {}
    for i, op in enumerate(k.ops):
        node = k.n_in + i
        if op[0] in ("cst", "zero"):
            depth[node] = 0
            continue
        if op[0] == "neg":
            src, n = slot_of[op[1]]
            slot_of[node] = (src, not n)
            depth[node] = depth[op[1]]
            continue
        assert op[0] in ("add", "sub", "mul", "fma", "fms", "fnma"), op
        depth[node] = 1 + max(depth[a] for a in op[1:])
        slot_of[node] = (nxt, False)
        nxt += 1
        per_level.setdefault(depth[node], []).append(i)
    assert nxt + 1 <= MAX_SLOTS
    D = max(per_level) if per_level else 0
    width = max((len(v) for v in per_level.values()), default=1)
    W = 1
    while W < width:
        W *= 2
    assert W <= 32, (R, twiddled, width)
    ONE, NZ = (0, False), (1, False)
    levels = []
    for L in range(1, D + 1):
        descs = []
        for i in per_level.get(L, []):
            op = k.ops[i]
            s = [slot_of[a] for a in op[1:]]
            o = op[0]
            neg = lambda v: (v[0], not v[1])
            if o == "add":
                A, B, C = s[0], ONE, s[1]
            elif o == "sub":
                A, B, C = neg(s[1]), ONE, s[0]
            elif o == "mul":
                A, B, C = s[0], s[1], NZ
            elif o == "fma":
                A, B, C = s[0], s[1], s[2]
            elif o == "fms":
                A, B, C = s[0], s[1], neg(s[2])
            else:  # fnma
                A, B, C = neg(s[0]), s[1], s[2]
            if B[1]:                                    # fma(a, -b, c) == fma(-a, b, c)
                A, B = neg(A), neg(B)
            descs.append(pack_desc(A[0], B[0], C[0], A[1], C[1], slot_of[k.n_in + i][0]))
        # idle lanes compute 1 * 1 + (-0) into a scratch slot (no divergence on the device)
        descs += [pack_desc(0, 0, 1, False, False, nxt)] * (W - len(descs))
        levels.append(tuple(descs))
    outs = tuple(slot_of[o][0] | (int(slot_of[o][1]) << 15) for o in k.outs)
    return WideSchedule(W, k.n_in, tuple(consts), tuple(levels), outs, nxt + 1)


def replay(ws: WideSchedule, fma, x: List[float]) -> List[float]:
    """Evaluate a schedule level by level with `fma(a, b, c)` (the host check of the tables)."""
    def f(b: int) -> float:
        return struct.unpack("<d", struct.pack("<Q", b))[0]
    V = [0.0] * ws.n_slots
    for i, c in enumerate(ws.consts):
        V[i] = f(c)
    for i, v in enumerate(x):
        V[ws.in_base + i] = v
    for lvl in ws.levels:
        res = []
        for d in lvl:
            u = unpack_desc(d)
            if u is None:
                continue
            a, b, c, na, nc, o = u
            res.append((o, fma(-V[a] if na else V[a], V[b], -V[c] if nc else V[c])))
        for o, v in res:                                # a level reads only earlier levels
            V[o] = v
    return [-V[o & 0x7fff] if o >> 15 else V[o] for o in ws.outs]


def c_tables(radices: List[int]) -> str:
    """The schedules of every (direction, radix, twiddled) as a C++ header: kWideInfo[fwd][R][tw]
    = {W, depth, n_in, n_consts, n_slots, desc offset, const offset, out offset}, then the
    descriptors, constants and output slots back to back (the planner copies a plan's
    schedules into the cluster kernel's device image)."""
    info = {}
    desc: List[int] = []
    cst: List[int] = []
    outs: List[int] = []
    for fwd in (False, True):
        for R in radices:
            for tw in (False, True):
                ws = wide_schedule(fwd, R, tw)
                info[(fwd, R, tw)] = (ws.W, ws.depth, ws.n_in, len(ws.consts), ws.n_slots,
                                      len(desc), len(cst), len(outs))
                for lvl in ws.levels:
                    desc.extend(lvl)
                cst.extend(ws.consts)
                outs.extend(ws.outs)
                # every block starts on a 16-byte boundary (the kernel copies them with
                # 16-byte asynchronous copies)
                desc.extend([0] * (len(desc) % 2))
                cst.extend([0] * (len(cst) % 2))
                outs.extend([0] * (-len(outs) % 4))
    head = ["// Generated by lfg/build.py from lfg/codegen/wide.py: lane-parallel schedules of the",
            "// binary64 butterflies (one operation per lane per level).",
            "#pragma once",
            "namespace lfg {",
            "struct WideInfo {",
            "  int W, depth, n_in, n_consts, n_slots, desc_off, const_off, out_off;",
            "};",
            "// [forward][R][twiddled]; W == 0: no schedule for that radix",
            "constexpr WideInfo kWideInfo[2][17][2] = {"]
    for fwd in (False, True):
        rows = []
        for R in range(17):
            cells = []
            for tw in (False, True):
                v = info.get((fwd, R, tw))
                cells.append("{" + ", ".join(map(str, v)) + "}" if v else "{0, 0, 0, 0, 0, 0, 0, 0}")
            rows.append("  {" + ", ".join(cells) + "}")
        head.append(" {" + ",\n".join(rows) + "},")
    head.append("};")
    head.append(f"constexpr int kWideMaxDepth = {max(v[1] for v in info.values())};")
    head.append(f"constexpr int kWideMaxSlots = {max(v[4] for v in info.values())};")
    head.append("}  // namespace lfg")

    def arr(name: str, ty: str, vals: List[int], per: int = 6) -> None:
        head.insert(-1, f"constexpr {ty} {name}[{len(vals)}] = {{")
        for i in range(0, len(vals), per):
            head.insert(-1, "  " + ", ".join(f"{v:#x}ull" if ty == "uint64_t" else f"{v}u"
                                             for v in vals[i:i + per]) + ",")
        head.insert(-1, "};")
    head.insert(3, "#include <cstdint>")
    arr("kWideDesc", "uint64_t", desc)
    arr("kWideConst", "uint64_t", cst)
    arr("kWideOut", "uint32_t", outs, 16)
    return "\n".join(head) + "\n"
