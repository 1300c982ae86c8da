"""Logging (the dolfinx.log calls): levels with the reference's values,
filtering, output to a file, the thread name in each line, timings at DEBUG
("Elapsed time"), and refused serving requests at WARNING."""

import logging
import sys

import pytest


@pytest.fixture
def log(capi, tmp_path):
    from dolfinx_gb300 import log as lg

    path = tmp_path / "run.log"
    old = lg.get_log_level()
    lg.set_output_file(str(path))
    pattern = lg._pattern
    yield lg, path
    lg.set_log_level(old)
    lg._pattern = pattern
    lg._install(logging.StreamHandler(sys.stderr))


def test_levels_have_the_reference_values(capi):
    from dolfinx_gb300 import log as lg

    names = ["TRACE", "DEBUG", "INFO", "WARNING", "ERROR", "CRITICAL", "OFF"]
    assert [lg.LogLevel[n].value for n in names] == list(range(7))


def test_filtering_and_output_file(log):
    lg, path = log
    assert lg.get_log_level() == lg.LogLevel.WARNING  # the default
    lg.log(lg.LogLevel.INFO, "hidden at WARNING")
    lg.log(lg.LogLevel.ERROR, "shown at WARNING")
    lg.set_log_level(lg.LogLevel.TRACE)
    assert lg.get_log_level() == lg.LogLevel.TRACE
    lg.log(lg.LogLevel.TRACE, "trace line")
    lg.log(lg.LogLevel.OFF, "never")
    lg.set_thread_name("worker-7")
    lg.log(lg.LogLevel.INFO, "named")
    text = path.read_text()
    assert "shown at WARNING" in text and "hidden" not in text
    assert "trace line" in text and "never" not in text
    assert "[worker-7] [INFO] named" in text


def test_timings_are_logged_at_debug(log):
    from dolfinx_gb300 import common

    lg, path = log
    lg.set_log_level(lg.LogLevel.DEBUG)
    t = common.Timer("logged task")
    t.stop()
    t.flush()
    assert "Elapsed time: " in path.read_text() and "(logged task)" in path.read_text()
    common.clear_timings()
