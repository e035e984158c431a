"""Regex-group balancing, as BitGen's entry script does it.

``balance_regex_groups`` follows ``scripts/run_bitgen.py:102-116``: regexes are sorted by a
"custom length" in which every ``\\xHH`` escape and every bracket class counts as one
character, then assigned greedily to the currently lightest group.  ``group_regex_in_list``
follows ``scripts/run_bitgen.py:71-88`` (group count capped at the number of regexes, empty
groups dropped, ``regex_group_number < 1`` meaning one regex per group).
"""

from __future__ import annotations

import re
from typing import List, Sequence


def regex_custom_length(regex: str) -> int:
    regex = re.sub(r"\\x[0-9A-Fa-f]{2}", "X", regex)
    regex = re.sub(r"\[[^\]]+\]", "Y", regex)
    return len(regex)


def balance_regex_groups(regex_list: List[str], regex_group_number: int) -> List[List[str]]:
    ordered = sorted(regex_list, key=regex_custom_length)
    groups: List[List[str]] = [[] for _ in range(regex_group_number)]
    loads = [0] * regex_group_number
    for r in ordered:
        i = loads.index(min(loads))
        groups[i].append(r)
        loads[i] += regex_custom_length(r)
    return groups


def group_regex_in_list(regex_list: Sequence[str], regex_group_number: int) -> List[List[str]]:
    regex_list = list(regex_list)
    if regex_group_number >= 1:
        regex_group_number = min(regex_group_number, len(regex_list))
        groups = balance_regex_groups(regex_list, regex_group_number)
    else:
        groups = [[r] for r in regex_list]
    return [g for g in groups if g]


def read_regex_file(path: str) -> List[str]:
    """``/regex/`` per line, as ``bitgen/tool/pcre.py:5-27`` reads PCRE files."""
    out = []
    with open(path) as f:
        for line in f:
            r = line.strip()
            if not r:
                continue
            a, b = r.find("/"), r.rfind("/")
            if a != 0 or b <= a:
                raise ValueError(f"Regex requires slashes: {r}")
            out.append(r[a + 1:b])
    return out
