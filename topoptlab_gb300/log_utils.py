"""Loggers with the reference interface (log_utils.py:147-381): verbosity
levels 10 debug, 15 perf, 20 info, 30 warning, 40 error, 50 critical; every
message is appended to ``<file>.log`` and echoed to stdout."""
from __future__ import annotations


def _noop(msg: str) -> None:
    return None


class EmptyLogger:
    def __call__(self, msg: str) -> None:
        return None

    debug = perf = info = warning = error = critical = staticmethod(_noop)


class SimpleLogger:
    def __init__(self, file: str, verbosity: int = 20) -> None:
        self.file = file if file.endswith(".log") else f"{file}.log"
        with open(self.file, "w"):
            pass
        levels = {"debug": 10, "perf": 15, "info": 20, "warning": 30, "error": 40, "critical": 50}
        for name, lvl in levels.items():
            if verbosity > lvl:
                setattr(self, name, _noop)

    def __call__(self, msg: str) -> None:
        self._write(msg)

    def _write(self, msg: str) -> None:
        if not msg.endswith("\n"):
            msg += "\n"
        with open(self.file, "a") as f:
            f.write(msg)
        print(msg, end="")

    def debug(self, msg: str) -> None:
        self._write("[DEBUG] " + msg)

    def perf(self, msg: str) -> None:
        self._write("[PERF] " + msg)

    def info(self, msg: str) -> None:
        self._write(msg)

    def warning(self, msg: str) -> None:
        self._write("[WARNING] " + msg)

    def error(self, msg: str) -> None:
        self._write("[ERROR] " + msg)

    def critical(self, msg: str) -> None:
        self._write("[CRITICAL] " + msg)
