"""The Node Editor's shared-memory channel (NodeEditorIpc_C.h) and the CPU side of live trees.

The channel is restated from the reference's NodeEditorIpc library (same object name, size and
message layout), so these tests play both ends in one process: one context stands for the
editor, another for the application.  Live-tree swaps that compile trees need a GPU and are in
tests/test_gpu_live.py; here only the rejection paths run."""
import os
import stat
import time

import pytest

NOT_INITIALISED, TOO_SMALL, NONE, SELECTED, IMPORT = -2, -1, 0, 1, 2


@pytest.fixture
def channels(native):
    fn = native
    try:
        editor, app = fn.EditorChannel(), fn.EditorChannel()
    except OSError as e:
        pytest.skip(f"no POSIX shared memory here: {e}")
    yield editor, app
    app.close()
    editor.close()


def test_selected_and_import_messages(channels):
    editor, app = channels
    assert app.poll() == (NONE, None)
    assert editor.send_selected("DQAF@BCQgM")
    assert app.poll() == (SELECTED, "DQAF@BCQgM")
    assert app.poll() == (NONE, None)                     # consumed
    assert editor.poll() == (NONE, None)                  # a sender does not read its own message
    assert app.send_import("BwA")
    assert editor.poll() == (IMPORT, "BwA")
    assert app.poll() == (NONE, None)


def test_newest_message_wins(channels):
    editor, app = channels
    for s in ("AAA", "BBB", "CCC"):
        editor.send_selected(s)
    assert app.poll() == (SELECTED, "CCC")
    assert app.poll() == (NONE, None)


def test_buffer_too_small_and_limits(native, channels):
    editor, app = channels
    editor.send_selected("X" * 100)
    assert app.poll(size=10)[0] == TOO_SMALL              # consumed, as in the reference
    assert app.poll() == (NONE, None)
    editor.send_selected("Y" * 20)
    assert app.poll(size=0)[0] == TOO_SMALL               # no buffer: left for the next poll
    assert app.poll() == (SELECTED, "Y" * 20)
    assert not editor.send_selected("Z" * (64 * 1024 - 3))  # does not fit with its header
    assert editor.send_selected("Z" * (64 * 1024 - 4))
    t, s = app.poll()
    assert t == SELECTED and len(s) == 64 * 1024 - 4
    L = native.lib()
    assert L.fnEditorIpcPollMessage(None, None, 0) == NOT_INITIALISED
    assert not L.fnEditorIpcSendSelectedNode(None, b"A")


def test_read_previous(native, channels):
    editor, _ = channels
    editor.send_selected("PREV")
    late = native.EditorChannel(read_previous=True)
    fresh = native.EditorChannel(read_previous=False)
    try:
        assert late.poll() == (SELECTED, "PREV")
        assert fresh.poll() == (NONE, None)
    finally:
        late.close()
        fresh.close()


def test_start_node_editor_with_a_stand_in(native, tmp_path):
    """StartNodeEditor runs the configured executable with the reference's arguments."""
    log = tmp_path / "args.txt"
    exe = tmp_path / "NodeEditor"
    exe.write_text(f"#!/bin/sh\necho \"$@\" > {log}\n")
    exe.chmod(exe.stat().st_mode | stat.S_IEXEC)
    native.set_node_editor_path(str(exe))
    try:
        assert native.start_node_editor("DQAF@BCQgM", detached=True, child=True)
        for _ in range(200):
            if log.exists() and log.read_text().strip():
                break
            time.sleep(0.025)
        assert log.read_text().split() == ["--detached", "--import-ent", "DQAF@BCQgM"]
        native.set_node_editor_path(str(tmp_path / "missing"))
        assert not native.start_node_editor(None, False, True)
    finally:
        native.set_node_editor_path(None)


def test_live_tree_rejects_bad_trees_without_a_current_one(native, channels):
    editor, app = channels
    live = native.LiveTree(app, None, dims=(3,), poll_ms=0)
    try:
        assert live.acquire() == (None, 0)
        assert live.update() == 0
        editor.send_selected("not a tree!")
        assert live.update() == -1                        # FN_ERR_ARG: does not decode
        info = live.info()
        assert info["rejected"] == 1 and info["lastStatus"] == -1 and "decode" in info["lastError"]
        assert live.acquire() == (None, 0)
        editor.send_import("DQAF@BCQgM")                  # import requests are for the editor
        assert live.update() == 0 and live.info()["rejected"] == 1
    finally:
        live.close()


def test_live_tree_argument_checks(native):
    L = native.lib()
    import ctypes
    dims = (ctypes.c_int * 1)(5)
    assert not L.fnLiveTreeCreate(None, None, dims, 1, 0)
    assert not L.fnLiveTreeCreate(None, None, None, 1, 0)
    assert L.fnLiveTreeUpdate(None) == -1
    assert not L.fnLiveTreeAcquire(None, None)
    L.fnLiveTreeDelete(None)
