"""INI configuration with command-line overrides, mirroring the reference's
Config (src/config.h:51-83, src/config.cpp:78-150, 255-297).

File format: a line starting with '[' opens the section named by its first
word less that word's last character (`[ns]` -> ns, as the reference's
sscanf reads it); `key = value` (separators space, '=' or tab) inside a
section; lines starting with '#' or ';' and text after ';' are comments.
`rewrite(argv)` applies `--section:key=value` overrides.  `get(section, key,
default)` converts to the default's type the way a C++ stream reads it (the
longest numeric prefix, 0 when there is none).
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
        for line in text.split("\n"):
            if line.startswith("["):
                # sscanf(buf, "[%4000s]", section): the first word after '['
                # (leading blanks skipped), its last character dropped
                words = line[1:].split()
                if words:
                    cur = self.data.setdefault(words[0][:4000][:-1], {})
                    continue
            if line.startswith("#") or line.startswith(";"):
                continue
            if cur is None:
                continue
            if line.endswith("\r"):
                line = line[:-1]
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
            # stream extraction: the longest decimal prefix, 0 when there is none
            m = _FLOAT.match(v)
            return float(m.group(1)) if m else 0.0
        return v


_FLOAT = re.compile(r"\s*([+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)")
