"""lb.in, read with the rules of the reference's parser (src/module_input.f90).

The Fortran host of laboetie keeps its own parser; this restatement lets a Python host, the
benchmark and the tests read the same files the same way:

* each line is read as 100 characters (longer lines are cut), left-adjusted and trimmed
  (module_input.f90:580-583);
* everything from the first '#' on is blanked, then the line is trimmed again (:591-602);
* blank lines are dropped (:604-611);
* a tag matches the first line whose first len(tag) characters are the tag and whose next
  character is a blank (or the line ends there), e.g. ``f_ext = 0 0 0``; the value is read
  list-directed from characters len(tag)+4 .. len(tag)+50 of that line, i.e. after
  ``tag = `` (input_dp :62-77, input_dp3, input_int, input_log :385-426, input_char :430-452);
* a logical is true if the first character read is T or t, false if F or f, else an error; a
  value that does not read as the tag's type is an error (the reference's READ fails).

A missing tag gives the caller's default, or raises as the reference stops.
"""
from __future__ import annotations

import os
import re

LINE_LEN = 100


class LbInError(ValueError):
    pass


def _clean_lines(text: str) -> list[str]:
    out = []
    for raw in text.splitlines():
        line = raw.expandtabs(1)[:LINE_LEN].strip()
        k = line.find("#")
        if k >= 0:
            line = line[:k]
        line = line.strip()
        if line:
            out.append(line)
    return out


def _list_directed(field: str) -> list[str]:
    """The items of a Fortran list-directed read: separated by blanks or commas, a '/' ends the
    record."""
    field = field.split("/")[0]
    return [t for t in re.split(r"[\s,]+", field.strip()) if t]


def _real(tok: str) -> float:
    try:
        return float(tok.replace("d", "e").replace("D", "e"))
    except ValueError:
        raise LbInError(f"cannot read a real from {tok!r}") from None


def _int(tok: str) -> int:
    try:
        return int(tok)
    except ValueError:
        raise LbInError(f"cannot read an integer from {tok!r}") from None


class LbIn:
    """The tags of one lb.in file."""

    def __init__(self, text: str):
        self.lines = _clean_lines(text)

    @classmethod
    def read(cls, path: str) -> "LbIn":
        if not os.path.exists(path):
            raise LbInError(f"Error opening file {path}")
        with open(path) as fh:
            return cls(fh.read())

    def _field(self, tag: str):
        j = len(tag)
        for line in self.lines:
            padded = line.ljust(j + 50)
            if padded[:j] == tag and padded[j] == " ":
                return padded[j + 3:j + 50]
        return None

    def _items(self, tag, n, conv, default):
        field = self._field(tag)
        if field is None:
            if default is None:
                raise LbInError(f"I could not find keyword '{tag}' in lb.in")
            return default
        items = _list_directed(field)
        if len(items) < n:
            raise LbInError(f"{tag}: expected {n} value(s), read {items!r}")
        vals = [conv(t) for t in items[:n]]
        return vals[0] if n == 1 else tuple(vals)

    def dp(self, tag, default=None):
        return self._items(tag, 1, _real, default)

    def dp3(self, tag, default=None):
        return self._items(tag, 3, _real, default)

    def int(self, tag, default=None):
        return self._items(tag, 1, _int, default)

    def int3(self, tag, default=None):
        return self._items(tag, 3, _int, default)

    def log(self, tag, default=None):
        field = self._field(tag)
        if field is None:
            if default is None:
                raise LbInError(f"I could not find keyword '{tag}' in lb.in")
            return default
        items = _list_directed(field)
        c = items[0].strip("'\"")[:1] if items else ""
        if c in ("T", "t"):
            return True
        if c in ("F", "f"):
            return False
        raise LbInError(f'Problem with logical tag "{tag}" in lb.in')

    def char(self, tag, default=None):
        field = self._field(tag)
        if field is None:
            if default is None:
                raise LbInError(f"I could not find keyword '{tag}' in lb.in")
            return default
        items = _list_directed(field)
        if not items:
            raise LbInError(f"I found nothing after sign = for {tag}")
        return items[0].strip("'\"")[:50]

    def flow_params(self) -> dict:
        """The tags the flow phase reads, with the reference's defaults: box (lx, ly, lz),
        geometryLabel, relaxation_time (module_collision.f90:38, default 1), target_error
        (equilibration.f90:57, default 1e-10), f_ext (:379, default 0), initialSolventDensity
        (init_simu.f90:31, default 1)."""
        return dict(lx=self.int("lx"), ly=self.int("ly"), lz=self.int("lz"),
                    geometryLabel=self.int("geometryLabel"),
                    relaxation_time=self.dp("relaxation_time", 1.0),
                    target_error=self.dp("target_error", 1e-10),
                    f_ext=self.dp3("f_ext", (0.0, 0.0, 0.0)),
                    rho0=self.dp("initialSolventDensity", 1.0))
