"""SQLite table cache (schema 2.1.0) against files written and read by the
reference's own ``volumential/table_manager.py`` (fixtures made by
``tests/golden/make_table_cache_golden.py``)."""

import importlib.util
import os
import shutil

import numpy as np
import pytest

from volumential_gb300.table_manager import NearFieldInteractionTableManager

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = np.load(os.path.join(HERE, "golden", "table_cache_golden.npz"))
REF_DB = os.path.join(HERE, "golden", "table_cache_ref.sqlite")


def _gen():
    spec = importlib.util.spec_from_file_location(
        "_make_table_cache_golden", os.path.join(HERE, "golden", "make_table_cache_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_loads_tables_written_by_the_reference(tmp_path):
    db = tmp_path / "ref.sqlite"
    shutil.copy(REF_DB, db)
    with NearFieldInteractionTableManager(str(db), root_extent=1.0, read_only=True) as m:
        assert m.cache_schema_version == "2.1.0"
        for dim, ktype, q, level, _ in _gen().TABLES:
            t = m.load_saved_table(dim, ktype, q, source_box_level=level)
            ids, vals = t.get_reduced_table_data()
            tag = f"ref_{dim}_{ktype}_{q}_{level}"
            np.testing.assert_array_equal(ids, GOLD[tag + "_ids"])
            np.testing.assert_array_equal(vals, GOLD[tag + "_vals"])
            np.testing.assert_array_equal(t.mode_normalizers, GOLD[tag + "_nmlz"])
            assert t.is_built and t.source_box_extent == 0.5 ** level
            if ktype == "Helmholtz":
                assert t.k == 3.0 and np.iscomplexobj(vals)
            # through get_table: a hit, not recomputed
            t2, recomputed = m.get_table(dim, ktype, q, source_box_level=level)
            assert not recomputed
            np.testing.assert_array_equal(t2.get_reduced_table_data()[1], vals)
        with pytest.raises(RuntimeError, match="read-only"):
            m.get_table(3, "Laplace", 3)


def test_reference_reads_the_tables_this_package_writes():
    gen = _gen()
    assert str(GOLD["ours_schema_version"]) == "2.1.0"
    for dim, ktype, q, level, seed in gen.TABLES:
        t = gen.seeded_table(dim, ktype, q, level, seed + 100)
        ids, vals = t.get_reduced_table_data()
        tag = f"ours_{dim}_{ktype}_{q}_{level}"
        np.testing.assert_array_equal(GOLD[tag + "_ids"], ids)
        np.testing.assert_array_equal(GOLD[tag + "_vals"], vals)
        assert int(GOLD[tag + "_reduced"][0]) == 1
        np.testing.assert_array_equal(GOLD[tag + "_row"],
                                      [t.n_q_points, q, t.n_pairs, 13, 6])
        assert float(GOLD[tag + "_extent"]) == 0.5 ** level
        if ktype == "Helmholtz":
            assert float(GOLD[tag + "_k"]) == 3.0


def test_round_trip_and_guards(tmp_path):
    gen = _gen()
    db = str(tmp_path / "rt.sqlite")
    with NearFieldInteractionTableManager(db, root_extent=1.0) as m:
        for dim, ktype, q, level, seed in gen.TABLES:
            m.store_table(gen.seeded_table(dim, ktype, q, level, seed), ktype, level)
    with NearFieldInteractionTableManager(db, root_extent=1.0) as m:
        for dim, ktype, q, level, seed in gen.TABLES:
            a = gen.seeded_table(dim, ktype, q, level, seed).get_reduced_table_data()
            b = m.load_saved_table(dim, ktype, q, level).get_reduced_table_data()
            np.testing.assert_array_equal(a[0], b[0])
            np.testing.assert_array_equal(a[1], b[1])
    with pytest.raises(RuntimeError, match="root_extent"):
        NearFieldInteractionTableManager(db, root_extent=2.0)
