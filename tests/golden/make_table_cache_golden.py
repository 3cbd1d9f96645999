"""Golden SQLite table caches, written and read by the reference's own code.

Run where the reference source tree is mounted (read only):

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_table_cache_golden.py /path/to/reference

``volumential/table_manager.py`` imports sumpy and the ``volumential``
package, which are absent here; this script executes the module from its
source path with three stand-in modules for those imports (an empty
``ExpressionKernel`` base class and empty packages), which the functions used
below never touch.  With the reference's own code it then:

1. creates a cache file (``NearFieldInteractionTableManager.__init__``:
   schema, ``schema_version`` and ``root_extent`` metadata), stores three
   seeded tables in it with the reference's payload serializer
   (``_serialize_table_payload``) and kwargs writer
   (``_store_record_kwargs``), the row values following
   ``_compute_and_update_table_for_request`` (``:1941-2060``) ->
   ``table_cache_ref.sqlite`` (read by this package's manager in the tests);
2. opens a cache written by this package's manager read-only and reads every
   row back with the reference's ``_load_record``, ``_deserialize_table_payload``
   and ``_load_record_kwargs``; the values it reads are saved for the test.

Outputs: ``table_cache_ref.sqlite`` and ``table_cache_golden.npz``.
"""

from __future__ import annotations

import importlib.util
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.dont_write_bytecode = True
sys.path.insert(0, ROOT)

TABLES = [(2, "Laplace", 2, 0, 11), (3, "Laplace", 2, 1, 12), (2, "Helmholtz", 2, 0, 13)]


def load_reference_table_manager(ref):
    stubs = {
        "sumpy": types.ModuleType("sumpy"),
        "sumpy.kernel": types.ModuleType("sumpy.kernel"),
        "volumential": types.ModuleType("volumential"),
        "volumential.nearfield_potential_table":
            types.ModuleType("volumential.nearfield_potential_table"),
    }
    stubs["sumpy.kernel"].ExpressionKernel = type("ExpressionKernel", (), {})
    stubs["volumential.nearfield_potential_table"].NearFieldInteractionTable = None
    saved = {k: sys.modules.get(k) for k in stubs}
    sys.modules.update(stubs)
    try:
        spec = importlib.util.spec_from_file_location(
            "_ref_table_manager", os.path.join(ref, "volumential", "table_manager.py"))
        tm = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(tm)
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    return tm


def seeded_table(dim, kernel_type, q, level, seed):
    from volumential_gb300.kernels import HelmholtzKernel, LaplaceKernel
    from volumential_gb300.nearfield_potential_table import NearFieldInteractionTable

    cplx = kernel_type == "Helmholtz"
    knl = HelmholtzKernel(dim) if cplx else LaplaceKernel(dim)
    t = NearFieldInteractionTable(q, dim=dim, sumpy_kernel=knl, source_box_extent=0.5 ** level,
                                  dtype=np.complex128 if cplx else np.float64)
    ids = t._get_invariant_entry_info()["entry_ids"]
    rng = np.random.default_rng(seed)
    vals = rng.standard_normal(len(ids))
    if cplx:
        vals = vals + 1j * rng.standard_normal(len(ids))
    t.set_reduced_table_data(ids, vals)
    if dim == 2:
        t.build_normalizer_table()
    return t


def main():
    if len(sys.argv) != 2:
        sys.exit(f"usage: python {sys.argv[0]} <path of the volumential source tree>")
    ref = sys.argv[1]
    tm = load_reference_table_manager(ref)
    from volumential_gb300.table_manager import NearFieldInteractionTableManager

    out = {}
    # 1. a cache written by the reference's code
    path = os.path.join(HERE, "table_cache_ref.sqlite")
    if os.path.exists(path):
        os.remove(path)
    mgr = tm.NearFieldInteractionTableManager(dataset_filename=path, root_extent=1.0,
                                              read_only=False)
    for dim, ktype, q, level, seed in TABLES:
        t = seeded_table(dim, ktype, q, level, seed)
        vals = sorted({int(c) for v in t.interaction_case_vecs for c in v})
        mgr.datafile.execute(
            "INSERT INTO nearfield_cache (dim, kernel_type, q_order, source_box_level, "
            "n_q_points, quad_order, n_pairs, source_box_extent, source_box_level_stored, "
            "case_encoding_base, case_encoding_shift, build_method, kernel_type_cached, "
            "payload) VALUES (?, ?, ?, ?, ?, ?, ?, ?, ?, ?, ?, ?, ?, ?)",
            (dim, ktype, q, level, t.n_q_points, t.quad_order, t.n_pairs,
             mgr._source_box_extent_for_level(level), level, vals[-1] - vals[0] + 1,
             -vals[0], "DuffyRadial", ktype, tm._serialize_table_payload(t)))
        req = tm.TableRequest.from_args(dim=dim, kernel_type=ktype, q_order=q,
                                        source_box_level=level)
        mgr._store_record_kwargs(req, {"k": 3.0} if ktype == "Helmholtz" else {})
        ids, data = t.get_reduced_table_data()
        out[f"ref_{dim}_{ktype}_{q}_{level}_ids"] = ids
        out[f"ref_{dim}_{ktype}_{q}_{level}_vals"] = data
        out[f"ref_{dim}_{ktype}_{q}_{level}_nmlz"] = np.array(t.mode_normalizers)
    mgr.datafile.commit()
    mgr.datafile.close()

    # 2. a cache written by this package, read by the reference's code
    with tempfile.TemporaryDirectory() as d:
        ours = os.path.join(d, "ours.sqlite")
        with NearFieldInteractionTableManager(ours, root_extent=1.0) as m:
            for dim, ktype, q, level, seed in TABLES:
                m.store_table(seeded_table(dim, ktype, q, level, seed + 100), ktype, level,
                              **({"k": 3.0} if ktype == "Helmholtz" else {}))
        rmgr = tm.NearFieldInteractionTableManager(dataset_filename=ours, root_extent=1.0,
                                                   read_only=True)
        out["ours_schema_version"] = np.array(str(rmgr.cache_schema_version))
        for dim, ktype, q, level, seed in TABLES:
            req = tm.TableRequest.from_args(dim=dim, kernel_type=ktype, q_order=q,
                                            source_box_level=level)
            row = rmgr._load_record(req)
            p = tm._deserialize_table_payload(row["payload"])
            kw = rmgr._load_record_kwargs(req)
            tag = f"ours_{dim}_{ktype}_{q}_{level}"
            out[tag + "_ids"] = p["reduced_entry_ids"]
            out[tag + "_vals"] = p["reduced_data"]
            out[tag + "_reduced"] = p["table_data_is_symmetry_reduced"]
            out[tag + "_row"] = np.array([row["n_q_points"], row["quad_order"], row["n_pairs"],
                                          row["case_encoding_base"],
                                          row["case_encoding_shift"]])
            out[tag + "_extent"] = np.array(row["source_box_extent"])
            out[tag + "_k"] = np.array(kw.get("k", np.nan))
        rmgr.datafile.close()
    np.savez_compressed(os.path.join(HERE, "table_cache_golden.npz"), **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
