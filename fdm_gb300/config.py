"""INI configuration with command-line overrides, mirroring the reference's
Config (src/config.h:51-83, src/config.cpp:78-150, 255-297).

File format: `[section]` lines open a section; `key = value` (separators
space, '=' or tab) inside a section; lines starting with '#' or ';' and text
after ';' are comments.  `rewrite(argv)` applies `--section:key=value`
overrides.  `get(section, key, default)` converts to the default's type.
"""
from __future__ import annotations

import re


class Config:
    def __init__(self):
        self.data: dict[str, dict[str, str]] = {}
        self.filename = ""

    def open(self, filename: str) -> None:
        self.filename = filename
        try:
            with open(filename, "r") as f:
                self.load(f.read())
        except OSError:
            return

    def load(self, text: str) -> None:
        cur = None
        for line in text.splitlines():
            m = re.match(r"\[(\S+)\]", line)
            if m:
                cur = self.data.setdefault(m.group(1), {})
                continue
            if line.startswith("#") or line.startswith(";"):
                continue
            if cur is None:
                continue
            line = line.split(";", 1)[0]
            toks = [t for t in re.split(r"[ =\t]+", line) if t]
            if len(toks) >= 2:
                cur[toks[0]] = toks[1]

    def rewrite(self, argv) -> None:
        for s in list(argv)[1:]:
            if not s.startswith("--"):
                continue
            s = s[2:]
            if ":" not in s:
                continue
            sec, rest = s.split(":", 1)
            if "=" not in rest:
                continue
            key, val = rest.split("=", 1)
            self.data.setdefault(sec, {})[key] = val

    def set(self, section: str, key: str, value) -> None:
        self.data.setdefault(section, {})[key] = str(value)

    def get(self, section: str, key: str, default):
        v = self.data.get(section, {}).get(key)
        if v is None:
            return default
        if isinstance(default, bool):
            return bool(int(v))
        if isinstance(default, int):
            m = re.match(r"\s*([+-]?\d+)", v)
            return int(m.group(1)) if m else 0
        if isinstance(default, float):
            return float(v)
        return v
