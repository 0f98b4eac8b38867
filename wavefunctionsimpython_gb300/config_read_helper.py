"""Dotted-path TOML parameter lookup (sources/config_read_helper.py:5-17).

Same semantics as the reference: walk ``a.b.c`` through nested tables and fall
back to the default with a printed warning when a key is missing. TOML files
are parsed with the standard library's ``tomllib``.
"""
from __future__ import annotations

import sys
import tomllib
from typing import Any, Dict

_RED = "\033[31m"
_RESET = "\033[0m"
QUIET = False


def try_read_param(config: Dict, tokens: str, default_val: Any, reached_tokens: str = ""):
    for token in tokens.split("."):
        try:
            config = config[token]
        except (KeyError, TypeError):
            if not QUIET:
                print(f"{_RED}Did not found token \"{token}\" under \"{reached_tokens}\"!\n"
                      f"Falling back to the default value of {default_val}.\n{_RESET}", file=sys.stderr)
            return default_val
        reached_tokens += ("." if len(reached_tokens) > 0 else "") + token
    return config


def load_toml(path) -> Dict:
    """Parses a configuration file; raises ``ValueError`` on malformed TOML
    (the reference prints and exits, sources/initialisation.py:44-49)."""
    with open(path, "rb") as f:
        try:
            return tomllib.load(f)
        except tomllib.TOMLDecodeError as e:
            raise ValueError(f"Failed to decode TOML file {path}: {e}") from e
