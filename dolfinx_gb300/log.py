"""Logging: the ``dolfinx.log`` calls (python/dolfinx/wrappers/log.cpp:19-95)
over Python's ``logging``, one logger named ``dolfinx_gb300`` writing plain
lines to stderr (or to a file after ``set_output_file``).

- ``LogLevel``: TRACE, DEBUG, INFO, WARNING, ERROR, CRITICAL, OFF with the
  values the reference's enum takes from spdlog;
- ``set_log_level`` / ``get_log_level``; the default is WARNING;
- ``log(level, message)``;
- ``set_output_file(filename)``, ``set_thread_name(name)``.

The package logs timings at DEBUG ("Elapsed time: ... (task)", as
TimeLogger::register_timing does) and refused serving requests at WARNING.
"""

from __future__ import annotations

import enum
import logging
import sys

__all__ = ["LogLevel", "get_log_level", "log", "set_log_level", "set_output_file",
           "set_thread_name"]


class LogLevel(enum.IntEnum):
    TRACE = 0
    DEBUG = 1
    INFO = 2
    WARNING = 3
    ERROR = 4
    CRITICAL = 5
    OFF = 6


# LogLevel -> logging level (TRACE below DEBUG; OFF above everything)
_TO_PY = {LogLevel.TRACE: 5, LogLevel.DEBUG: logging.DEBUG, LogLevel.INFO: logging.INFO,
          LogLevel.WARNING: logging.WARNING, LogLevel.ERROR: logging.ERROR,
          LogLevel.CRITICAL: logging.CRITICAL, LogLevel.OFF: logging.CRITICAL + 10}
_FROM_PY = {v: k for k, v in _TO_PY.items()}

logger = logging.getLogger("dolfinx_gb300")
logger.propagate = False
_pattern = "[%(asctime)s] [%(threadName)s] [%(levelname)s] %(message)s"


def _install(handler: logging.Handler) -> None:
    for h in list(logger.handlers):
        logger.removeHandler(h)
        h.close()
    handler.setFormatter(logging.Formatter(_pattern))
    logger.addHandler(handler)


_install(logging.StreamHandler(sys.stderr))
logger.setLevel(_TO_PY[LogLevel.WARNING])


def set_log_level(level: LogLevel) -> None:
    """Messages below `level` are dropped."""
    logger.setLevel(_TO_PY[LogLevel(level)])


def get_log_level() -> LogLevel:
    return _FROM_PY.get(logger.level, LogLevel.WARNING)


def log(level: LogLevel, message: str) -> None:
    """Log `message` at `level` (OFF logs nothing)."""
    level = LogLevel(level)
    if level != LogLevel.OFF:
        logger.log(_TO_PY[level], message)


def set_output_file(filename: str) -> None:
    """Send the log to `filename` (appended) instead of stderr."""
    _install(logging.FileHandler(filename))


def set_thread_name(thread_name: str) -> None:
    """Show `thread_name` in place of Python's thread name in every line."""
    global _pattern
    name = thread_name.replace("%", "%%")
    _pattern = f"[%(asctime)s] [{name}] [%(levelname)s] %(message)s"
    for h in logger.handlers:
        h.setFormatter(logging.Formatter(_pattern))
