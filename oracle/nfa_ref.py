"""Independent regex oracle: byte-level Thompson NFA simulation (test infrastructure only).

It shares nothing with the bitstream compiler except the regex parser: the parsed regex is
turned into an epsilon-NFA and simulated position by position, injecting the start state at
every position (matches may start anywhere).  Bit ``p`` of the result is set iff some non-empty
match ends with the byte at ``p``.  ``^`` holds at position 0 and after an LF; ``$`` holds before
an LF and at the end of the input; ``\\A`` at position 0, ``\\z`` at the end of the input and
``\\Z`` there or before a final LF; a lookaround when its own NFA matches from (ahead) or up to
(behind) that gap.  This is the
match-end convention stated in ``bitgen_gb300.regex`` for BitGen's count check against icgrep
(``bitgen/from_icgrep.py:59-121``): the count of a group is the popcount of the OR of its
regexes' streams (``bitgen/bitstream.py:60-61``).
"""

from __future__ import annotations

from bitgen_gb300.regex import (CC, WORD, Alt, End, Look, Rep, Seq, Start, TextEnd, TextStart,
                                WordB, parse_regex)

LF = 0x0A


class _NFA:
    def __init__(self):
        self.kind = []   # 'eps' | 'cc' | 'acc' | 'look' | an assertion: sol eol wb nwb sot eot eotz
        self.arg = []    # byte set for 'cc'
        self.out = []    # list of successor ids

    def new(self, kind, arg=None):
        self.kind.append(kind)
        self.arg.append(arg)
        self.out.append([])
        return len(self.kind) - 1

    def frag(self, node):
        """Return (entry, exit) state ids; exit is an 'eps' state with no successors yet."""
        if isinstance(node, CC):
            a = self.new("cc", node.bytes_)
            e = self.new("eps")
            self.out[a].append(e)
            return a, e
        assertion = {End: "eol", Start: "sol", TextStart: "sot"}.get(type(node))
        if isinstance(node, WordB):
            assertion = "nwb" if node.neg else "wb"
        if isinstance(node, TextEnd):
            assertion = "eotz" if node.final_lf else "eot"
        if isinstance(node, Look):      # its own NFA, run at the gap when the state is reached
            a = self.new("look", (_build(node.item), node.behind, node.neg))
            e = self.new("eps")
            self.out[a].append(e)
            return a, e
        if assertion is not None:     # a zero-width state passed when its condition holds
            a = self.new(assertion)
            e = self.new("eps")
            self.out[a].append(e)
            return a, e
        if isinstance(node, Seq):
            a = self.new("eps")
            cur = a
            for it in node.items:
                s, e = self.frag(it)
                self.out[cur].append(s)
                cur = e
            return a, cur
        if isinstance(node, Alt):
            a = self.new("eps")
            e = self.new("eps")
            for it in node.items:
                s, x = self.frag(it)
                self.out[a].append(s)
                self.out[x].append(e)
            return a, e
        if isinstance(node, Rep):
            a = self.new("eps")
            cur = a
            for _ in range(node.lo):
                s, x = self.frag(node.item)
                self.out[cur].append(s)
                cur = x
            if node.hi is None:
                s, x = self.frag(node.item)
                loop = self.new("eps")
                self.out[cur].append(loop)
                self.out[loop].append(s)
                self.out[x].append(loop)
                e = self.new("eps")
                self.out[loop].append(e)
                return a, e
            e = self.new("eps")
            for _ in range(node.hi - node.lo):
                s, x = self.frag(node.item)
                self.out[cur].append(s)
                self.out[cur].append(e)
                cur = x
            self.out[cur].append(e)
            return a, e
        raise TypeError(node)


class _Sim:
    """Simulation of one NFA over one input.  A lookaround state holds its own NFA (``arg``) and
    is passed at a gap when that NFA matches there: ahead, a match starting at the gap; behind,
    a match ending at it (possibly empty, both)."""

    def __init__(self, nfa: "_NFA", start: int, acc: int, data: bytes):
        self.nfa, self.start, self.acc, self.data, self.n = nfa, start, acc, data, len(data)
        self._ends = None          # gaps where a match ends (lookbehind)
        self._subs = {}

    def word(self, q):   # positions outside the input are non-word
        return 0 <= q < self.n and self.data[q] in WORD

    def sub(self, s):
        if s not in self._subs:
            sub_nfa, sub_start, sub_acc = self.nfa.arg[s][0]
            self._subs[s] = _Sim(sub_nfa, sub_start, sub_acc, self.data)
        return self._subs[s]

    def holds(self, s, gap) -> bool:
        _, behind, neg = self.nfa.arg[s]
        sim = self.sub(s)
        ok = sim.ends_at(gap) if behind else sim.starts_at(gap)
        return ok != neg

    def closure(self, states, gap):
        """Epsilon closure at the gap before byte ``gap`` (0 .. n)."""
        data, n = self.data, self.n
        holds = {"eps"}
        if gap == 0 or data[gap - 1] == LF:
            holds.add("sol")
        if gap == n or data[gap] == LF:
            holds.add("eol")
        holds.add("wb" if self.word(gap - 1) != self.word(gap) else "nwb")
        if gap == 0:
            holds.add("sot")
        if gap == n or (gap == n - 1 and data[gap] == LF):
            holds.add("eotz")
            if gap == n:
                holds.add("eot")
        seen = set()
        stack = list(states)
        while stack:
            s = stack.pop()
            if s in seen:
                continue
            seen.add(s)
            k = self.nfa.kind[s]
            if k in holds or (k == "look" and self.holds(s, gap)):
                stack.extend(self.nfa.out[s])
        return seen

    def step(self, active, p):
        byte = self.data[p]
        nxt = set()
        for s in active:
            if self.nfa.kind[s] == "cc" and byte in self.nfa.arg[s]:
                nxt.update(self.nfa.out[s])
        return nxt

    def starts_at(self, gap) -> bool:
        """Some match (possibly empty) starts at the gap."""
        cur = self.closure({self.start}, gap)
        for p in range(gap, self.n + 1):
            if self.acc in cur:
                return True
            if not cur or p == self.n:
                return False
            cur = self.closure(self.step(cur, p), p + 1)
        return False

    def ends_at(self, gap) -> bool:
        """Some match (possibly empty) ends at the gap."""
        if self._ends is None:
            ends = set()
            cur = set()
            for p in range(self.n + 1):
                cur = self.closure(cur | {self.start}, p)
                if self.acc in cur:
                    ends.add(p)
                if p < self.n:
                    cur = self.step(cur, p)
            self._ends = ends
        return gap in self._ends

    def match_ends(self) -> int:
        result = 0
        cur = set()
        for p in range(self.n):
            active = self.closure(cur | {self.start}, p)
            cur = self.closure(self.step(active, p), p + 1)
            if self.acc in cur:
                result |= 1 << p
        return result


def _build(node):
    nfa = _NFA()
    start, end = nfa.frag(node)
    acc = nfa.new("acc")
    nfa.out[end].append(acc)
    return nfa, start, acc


def match_ends(regex: str, data: bytes) -> int:
    """Match-end stream of ``regex`` over ``data`` as a big int (bit p = position p)."""
    nfa, start, acc = _build(parse_regex(regex))
    return _Sim(nfa, start, acc, data).match_ends()


def group_match_ends(regexes, data: bytes) -> int:
    r = 0
    for x in regexes:
        r |= match_ends(x, data)
    return r
