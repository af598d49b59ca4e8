"""The C-ABI library loads and exports every entry point include/ declares (no GPU call)."""
import ctypes
import re

from conftest import ROOT


def test_library_exports_declared_symbols():
    from strobealign_gb300 import build
    lib_path = build.library_path()
    if not lib_path.exists():
        build.build()
    lib = ctypes.CDLL(str(lib_path))
    header = (ROOT / "include" / "strobealign_gb300.h").read_text()
    names = sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(sa_[a-z_0-9]+)\(", header, re.M)))
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from strobealign_gb300 import _lib
    header = (ROOT / "include" / "strobealign_gb300.h").read_text()
    names = set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(sa_[a-z_0-9]+)\(", header, re.M))
    assert names <= set(_lib.SIGNATURES), names - set(_lib.SIGNATURES)


def test_version_and_defaults_without_gpu():
    import strobealign_gb300 as sa
    assert b"strobealign" in sa.lib().sa_version()
    p = sa.SeedingParameters.from_read_length(150)
    assert (p.k, p.s, p.w_min, p.w_max, p.max_dist) == (20, 16, 5, 11, 80)
    assert p.main_hash_mask == 0xFFFFFFFFFC000000 and p.partial_orientation_pos == 25
    # src/seeding/parameters.rs:334-373: read length 251 takes the 250 profile
    p = sa.SeedingParameters.from_read_length(251)
    assert (p.k, p.s, p.w_min, p.w_max, p.max_dist, p.q) == (22, 18, 6, 16, 180, 255)
    assert p.main_hash_mask == 0xFFFFFFFFFC000000 and p.partial_orientation_pos == 25
    assert p.forward_main_hash_mask == 0xFFFFFFFFFC000000 | (1 << 25)
    # :376-383: read lengths next to a profile's take its parameters
    fields = [f for f, _ in type(p.c)._fields_]
    as_tuple = lambda rl: tuple(getattr(sa.SeedingParameters.from_read_length(rl).c, f) for f in fields)
    assert as_tuple(149) == as_tuple(150) == as_tuple(151)
    m = sa.mapping_defaults()
    assert (m.max_tries, m.rescue_distance, m.match, m.mismatch, m.gap_open, m.gap_extend, m.end_bonus) == \
        (20, 100, 2, 8, 12, 1, 10)
    # session defaults: arena and reserve sized from free device memory at creation,
    # two admission lanes, batches copied at submit
    from strobealign_gb300 import _lib as L
    sp = L.SessionParams()
    sa.lib().sa_session_params_default(ctypes.byref(sp))
    assert (sp.max_inflight_bases, sp.max_inflight_requests, sp.policy_threads, sp.admission_streams,
            sp.borrow_inputs, sp.device_reserve_bytes) == (0, 0, 0, 2, 0, 0)
    assert ctypes.sizeof(L.SessionParams) == 32
    # batch schedule defaults: eight NAM parts, overlapped
    sc = L.ScheduleParams()
    sa.lib().sa_schedule_params_default(ctypes.byref(sc))
    assert (sc.parts, sc.overlap, sc.wave_min_jobs, sc.max_wave_jobs) == (8, 1, 32768, 262144)


def test_synthetic_generator_is_deterministic():
    from strobealign_gb300 import synthetic as syn
    g1 = syn.make_genome(3, 20000, 2, gc=0.41, segdup_fraction=0.1)
    g2 = syn.make_genome(3, 20000, 2, gc=0.41, segdup_fraction=0.1)
    assert all((a == b).all() for a, b in zip(g1.seqs, g2.seqs))
    a1, a2 = syn.make_paired_end(4, g1, 50)
    b1, b2 = syn.make_paired_end(4, g1, 50)
    assert (a1.seq == b1.seq).all() and (a2.seq == b2.seq).all()
