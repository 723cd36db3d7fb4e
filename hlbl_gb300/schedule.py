"""The sliding-hypercube schedule (src/schedule.cpp of the reference): which
sources are solved, in which order, and which pairs each new source closes.

Pure host logic; the batched path contracts each Source's partners in one
launch, so it needs these lists. Tests check them against the reference's
own build_schedule/simulate output (tests/golden).
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Tuple

Vec4 = Tuple[int, int, int, int]


def _add(a, b):
    return tuple(x + y for x, y in zip(a, b))


def _sub(a, b):
    return tuple(x - y for x, y in zip(a, b))


def _scale(s, a):
    return tuple(s * x for x in a)


def mod_pos(a, L):
    """a mod L in [0, L) per direction (vec4.hpp:17-24)."""
    return tuple(x % l for x, l in zip(a, L))


def site_map(x, L):
    """[0, L) -> [-L/2, L/2) (vec4.hpp:29-33)."""
    return tuple(v - l if v >= l // 2 else v for v, l in zip(x, L))


def site_map_diff(a, b, L):
    """Minimum-image a - b (vec4.hpp:38-40)."""
    return site_map(mod_pos(_sub(a, b), L), L)


def sign_vectors() -> List[Vec4]:
    """The 16 sign vectors in the reference's order (schedule.cpp:34-47)."""
    return [(a, b, c, d) for a in (-1, 1) for b in (-1, 1) for c in (-1, 1) for d in (-1, 1)]


def window_offsets(h) -> List[Vec4]:
    """{0} u (G minus h) in solve order, reflected by h (schedule.cpp:49-59)."""
    out = [(0, 0, 0, 0)]
    for g in sign_vectors():
        if g == (1, 1, 1, 1):
            continue
        out.append(tuple(hh * gg for hh, gg in zip(h, g)))
    return out


@dataclass
class Source:
    position: Vec4
    partners: List[Vec4] = field(default_factory=list)


@dataclass
class Step:
    index: int
    sources: List[Source] = field(default_factory=list)

    @property
    def n_pairs(self) -> int:
        return sum(len(s.partners) for s in self.sources)


def _is_diag(d, stride) -> bool:
    return all(abs(x) == stride for x in d)


def build_schedule(h, stride: int, n_steps: int, origin=(0, 0, 0, 0)) -> List[Step]:
    """Windows 0..n_steps (schedule.cpp:61-91)."""
    offsets = window_offsets(h)
    steps, prev = [], []
    for k in range(n_steps + 1):
        window = [_add(origin, _scale(stride, _add(_scale(k, h), a))) for a in offsets]
        available = list(prev)
        step = Step(index=k)
        for p in window:
            if p in available:
                continue
            src = Source(position=p, partners=[q for q in available if _is_diag(_sub(p, q), stride)])
            step.sources.append(src)
            available.append(p)
        steps.append(step)
        prev = window
    return steps


def all_pairs(steps) -> List[Tuple[Vec4, Vec4, int]]:
    """(older, newer, window) of every pair in schedule order (schedule.cpp:101-109)."""
    return [(q, s.position, st.index) for st in steps for s in st.sources for q in s.partners]


def simulate(steps, interleaved: bool = True):
    """(propagators, pairs, peak cache) without computing (schedule.cpp:168-214)."""
    pending = {}
    for older, newer, _ in all_pairs(steps):
        pending[older] = pending.get(older, 0) + 1
        pending[newer] = pending.get(newer, 0) + 1
    cache, peak, n_prop, n_pairs = set(), 0, 0, 0

    def contract(older, newer):
        nonlocal n_pairs
        n_pairs += 1
        for p in (older, newer):
            pending[p] -= 1
            if pending[p] == 0:
                cache.discard(p)

    for st in steps:
        if interleaved:
            for s in st.sources:
                cache.add(s.position)
                n_prop += 1
                peak = max(peak, len(cache))
                for q in s.partners:
                    contract(q, s.position)
        else:
            for s in st.sources:
                cache.add(s.position)
                n_prop += 1
                peak = max(peak, len(cache))
            for s in st.sources:
                for q in s.partners:
                    contract(q, s.position)
    if cache:
        raise RuntimeError("simulate: propagators left in the cache after the last pair")
    return n_prop, n_pairs, peak


@dataclass
class Plan2p2:
    """Which solves are followed by 2+2 (schedule.hpp:93-103): the first solve,
    over the chains in order (windows, then solve order), of each 2+2 source,
    sites compared wrapped onto the lattice."""
    at: List[dict] = field(default_factory=list)           # per chain: position -> source index
    not_sources: List[Tuple[Vec4, int, int]] = field(default_factory=list)  # (site, chain, window)
    unsolved: List[int] = field(default_factory=list)     # indices of sources no chain solves


def plan_2p2(chains, sources, lattice) -> Plan2p2:
    """schedule.cpp:284-313."""
    index = {}
    for i, s in enumerate(sources):
        index.setdefault(mod_pos(s, lattice), i)
    plan = Plan2p2(at=[{} for _ in chains])
    solved = set()
    for c, chain in enumerate(chains):
        for st in chain:
            for src in st.sources:
                p = mod_pos(src.position, lattice)
                if p in solved:
                    continue
                solved.add(p)
                if p in index:
                    plan.at[c][tuple(src.position)] = index[p]
                else:
                    plan.not_sources.append((p, c, st.index))
    plan.unsolved = [i for i, s in enumerate(sources) if mod_pos(s, lattice) not in solved]
    return plan


def report_2p2(plan: Plan2p2, sources) -> List[str]:
    """The warnings about a plan (schedule.cpp:315-347), the same lines."""
    lines: List[str] = []
    if not sources:
        return lines
    max_sites = 10
    n_not = len(plan.not_sources)
    if n_not > 0:
        lines.append(f"WARNING: {n_not} solved source positions are not 2+2 sources (no 2+2 "
                     "computed for them)")
        for p, chain, window in plan.not_sources[:max_sites]:
            lines.append(f"  ({p[0]},{p[1]},{p[2]},{p[3]}) in window {window} of chain {chain}")
        if n_not > max_sites:
            lines.append(f"  ... and {n_not - max_sites} more")
    n_uns = len(plan.unsolved)
    if n_uns > 0:
        lines.append(f"WARNING: {n_uns} 2+2 sources are not solved by any chain (no 2+2 "
                     "computed for them)")
        for i in plan.unsolved[:max_sites]:
            p = sources[i]
            lines.append(f"  ({p[0]},{p[1]},{p[2]},{p[3]})")
        if n_uns > max_sites:
            lines.append(f"  ... and {n_uns - max_sites} more")
    return lines
