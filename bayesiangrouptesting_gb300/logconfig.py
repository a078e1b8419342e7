"""Process-wide logging settings with the reference's names
(include/bgt/logging.hpp:11-52; behaviour of src/runtime/logging.cpp).

A message is written when its level is at or below the configured level
(``off`` silences everything), its subsystem is listed (an empty list means
all) and, under torch.distributed, the rank is in ``rank_filter`` (empty:
every rank).  Lines go to ``file_path`` when set, else to stderr, as
``[timestamp ]LEVEL subsystem[ rank=r/w] file:line: message``.  The
environment variables BGT_LOG_LEVEL, BGT_LOG_SUBSYS, BGT_LOG_FILE,
BGT_LOG_RANKS, BGT_LOG_COLOR and BGT_PERF_LEVEL are applied once, on the first
read of the configuration.
"""
from __future__ import annotations

import copy
import enum
import inspect
import os
import sys
import threading
import time
from dataclasses import dataclass, field
from typing import List


class LogLevel(enum.IntEnum):
    off = 0
    fatal = 1
    error = 2
    warn = 3
    info = 4
    debug = 5
    trace = 6


class LogSubsystem(enum.IntEnum):
    core = 0
    model = 1
    tree = 2
    runtime = 3
    parallel = 4
    cuda = 5
    jit = 6
    perf = 7


@dataclass
class LogConfig:
    level: LogLevel = LogLevel.warn
    subsystems: List[LogSubsystem] = field(default_factory=list)
    rank_filter: List[int] = field(default_factory=list)
    color: bool = False
    timestamps: bool = True
    file_path: str = ""


_lock = threading.Lock()
_config = LogConfig()
_env_applied = False

_LEVEL_NAMES = {"off": LogLevel.off, "fatal": LogLevel.fatal, "error": LogLevel.error, "warn": LogLevel.warn,
                "warning": LogLevel.warn, "info": LogLevel.info, "debug": LogLevel.debug, "trace": LogLevel.trace}


def parse_log_level(value: str) -> LogLevel:
    """Case-insensitive level name; anything unknown is ``warn``."""
    return _LEVEL_NAMES.get(value.strip().lower(), LogLevel.warn)


def parse_log_subsystem(value: str) -> LogSubsystem:
    """Case-insensitive subsystem name; anything unknown is ``runtime``."""
    try:
        return LogSubsystem[value.strip().lower()]
    except KeyError:
        return LogSubsystem.runtime


def log_level_name(level: LogLevel) -> str:
    return LogLevel(level).name.upper()


def log_subsystem_name(subsystem: LogSubsystem) -> str:
    return LogSubsystem(subsystem).name


def _split(value: str) -> List[str]:
    return [part for part in value.split(",") if part]


def _apply_environment() -> None:
    global _env_applied
    if _env_applied:
        return
    _env_applied = True
    env = os.environ
    if "BGT_LOG_LEVEL" in env:
        _config.level = parse_log_level(env["BGT_LOG_LEVEL"])
    if "BGT_LOG_SUBSYS" in env:
        _config.subsystems = [parse_log_subsystem(p) for p in _split(env["BGT_LOG_SUBSYS"])]
    if "BGT_LOG_FILE" in env:
        _config.file_path = env["BGT_LOG_FILE"]
    if "BGT_LOG_RANKS" in env:
        _config.rank_filter = [int(p) for p in _split(env["BGT_LOG_RANKS"])]
    if "BGT_LOG_COLOR" in env:
        _config.color = env["BGT_LOG_COLOR"].lower() in ("1", "true", "on")
    if "BGT_PERF_LEVEL" in env:
        _config.level = max(_config.level, parse_log_level(env["BGT_PERF_LEVEL"]))
        if LogSubsystem.perf not in _config.subsystems:
            _config.subsystems.append(LogSubsystem.perf)


def set_log_config(config: LogConfig) -> None:
    global _config
    with _lock:
        _config = copy.deepcopy(config)


def get_log_config() -> LogConfig:
    with _lock:
        _apply_environment()
        return copy.deepcopy(_config)


def set_log_level(level: LogLevel) -> None:
    with _lock:
        _config.level = LogLevel(level)


def _rank():
    try:
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            return dist.get_rank(), dist.get_world_size()
    except Exception:
        pass
    return None


def log_enabled(level: LogLevel, subsystem: LogSubsystem) -> bool:
    with _lock:
        _apply_environment()
        cfg = _config
        if cfg.level == LogLevel.off or level == LogLevel.off:
            return False
        if int(level) > int(cfg.level):
            return False
        if cfg.subsystems and subsystem not in cfg.subsystems:
            return False
        if cfg.rank_filter:
            rank = _rank()
            if rank is not None and rank[0] not in cfg.rank_filter:
                return False
        return True


def log_message(level: LogLevel, subsystem: LogSubsystem, message: str) -> None:
    """Writes one line when the configuration enables it (the caller's file
    and line go into the prefix)."""
    if not log_enabled(level, subsystem):
        return
    frame = inspect.currentframe()
    caller = frame.f_back if frame is not None and frame.f_back is not None else None
    filename = caller.f_code.co_filename if caller is not None else "?"
    lineno = caller.f_lineno if caller is not None else 0
    del frame, caller
    with _lock:
        cfg = copy.deepcopy(_config)
    parts = []
    if cfg.timestamps:
        parts.append(time.strftime("%Y-%m-%d %H:%M:%S"))
    parts.append(f"{log_level_name(level)} {log_subsystem_name(subsystem)}")
    rank = _rank()
    if rank is not None:
        parts.append(f"rank={rank[0]}/{rank[1]}")
    parts.append(f"{os.path.basename(filename)}:{lineno}: {message}")
    line = " ".join(parts)
    if cfg.color and not cfg.file_path:
        colour = {LogLevel.fatal: 31, LogLevel.error: 31, LogLevel.warn: 33, LogLevel.info: 32}.get(level, 36)
        line = f"\033[{colour}m{line}\033[0m"
    if cfg.file_path:
        with _lock, open(cfg.file_path, "a", encoding="utf-8") as fh:
            fh.write(line + "\n")
    else:
        print(line, file=sys.stderr, flush=True)
