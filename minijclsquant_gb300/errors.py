"""How the drop-in modules report a missing or invalid argument.

By default they keep the reference's behaviour: print its message and return None
(jclsquant/recurrence_functions.py:11-13 and the like), so code written against the
reference sees the same thing.  In strict mode they raise ValueError with that message
instead, so a caller cannot go on with None by mistake.  Strict mode is on when the
environment variable KPM_STRICT_ERRORS is set to a nonzero value, after set_strict(True),
or inside ``with strict():``.
"""
from __future__ import annotations

import contextlib
import os

_strict = os.environ.get("KPM_STRICT_ERRORS", "") not in ("", "0")


def set_strict(on: bool) -> None:
    """Switch strict mode on (raise ValueError) or off (the reference's message and None)."""
    global _strict
    _strict = bool(on)


def is_strict() -> bool:
    return _strict


@contextlib.contextmanager
def strict(on: bool = True):
    """Strict mode (or, with on=False, the reference's behaviour) inside a with-block."""
    global _strict
    old = _strict
    _strict = bool(on)
    try:
        yield
    finally:
        _strict = old


def missing(message: str):
    """Report a missing or invalid argument: raise ValueError in strict mode, else print the
    reference's message and return None (the caller returns that value)."""
    if _strict:
        raise ValueError(message.strip())
    print(message)
    return None
