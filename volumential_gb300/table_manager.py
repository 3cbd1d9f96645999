"""SQLite table cache, compatible with the reference's cache files.

``NearFieldInteractionTableManager`` keeps the reference's interface
(``volumential/table_manager.py:521-1720``): ``get_table(dim, kernel_type,
q_order, source_box_level=0, force_recompute=False, queue=None, **kwargs)``
returns ``(table, is_recomputed)``, loading a stored table or building it
(here with the FP64 GPU builder) and storing it; ``load_saved_table`` loads
only.  The file format is the reference's cache schema 2.1.0, so caches are
shared both ways:

* table ``nearfield_cache``: one row per (dim, kernel_type, q_order,
  source_box_level) with the table's sizes, source box extent, the case
  encoding base/shift, build method and an ``npz`` payload
  (``:171-229``: q_points, mode_normalizers, kernel_exterior_normalizers,
  interaction_case_vecs, case_indices, table_data_is_symmetry_reduced, and
  either ``data`` or ``reduced_entry_ids`` + ``reduced_data``);
* table ``nearfield_cache_kwargs``: typed scalar build arguments per row
  (``:268-303`` serialisation: bool/int/float/complex/str);
* table ``nearfield_cache_meta``: ``schema_version`` and ``root_extent``.

Kernel types built here: Laplace, Helmholtz (wave number ``k``) and
Constant; rows of other kernel types load (their data is stored) with
``sumpy_kernel=None``.
"""

from __future__ import annotations

import logging
import sqlite3
import time
import zipfile
from io import BytesIO
from urllib.parse import quote

import numpy as np

from .kernels import ConstantKernel, HelmholtzKernel, LaplaceKernel
from .nearfield_potential_table import NearFieldInteractionTable

logger = logging.getLogger(__name__)

__all__ = ["NearFieldInteractionTableManager", "TABLE_CACHE_SCHEMA_VERSION"]

TABLE_CACHE_SCHEMA_VERSION = "2.1.0"
_BUILD_METHOD = "DuffyRadial"
_KERNELS = {"Laplace": LaplaceKernel, "Helmholtz": HelmholtzKernel,
            "Constant": ConstantKernel}


def _uri(path, mode):
    return "file:{}?mode={}".format(quote(str(path), safe="/"), mode)


def _scalar_to_text(value):
    if isinstance(value, (bool, np.bool_)):
        return "bool", str(int(value))
    if isinstance(value, (int, np.integer)):
        return "int", str(int(value))
    if isinstance(value, (float, np.floating)):
        return "float", repr(float(value))
    if isinstance(value, (complex, np.complexfloating)):
        return "complex", repr(complex(value))
    if isinstance(value, str):
        return "str", value
    raise TypeError(f"unsupported value type {type(value)!r}")


def _text_to_scalar(ty, text):
    conv = {"bool": lambda t: bool(int(t)), "int": int, "float": float, "complex": complex,
            "str": str}
    if ty not in conv:
        raise ValueError(f"unsupported serialized value type {ty}")
    return conv[ty](text)


def table_payload(table):
    """The row payload of a table (an ``npz`` archive)."""
    reduced = bool(getattr(table, "table_data_is_symmetry_reduced", False))
    arrays = {
        "q_points": np.array(table.q_points),
        "mode_normalizers": np.array(table.mode_normalizers),
        "kernel_exterior_normalizers": np.array(table.kernel_exterior_normalizers),
        "interaction_case_vecs": np.array(table.interaction_case_vecs),
        "case_indices": np.array(table.case_indices),
        "table_data_is_symmetry_reduced": np.array([int(reduced)], dtype=np.int8),
    }
    if getattr(table, "symmetry_source_direction", None) is not None:
        arrays["symmetry_source_direction"] = np.asarray(table.symmetry_source_direction,
                                                          dtype=np.float64)
    if reduced:
        ids, vals = table.get_reduced_table_data()
        arrays["reduced_entry_ids"] = np.asarray(ids, dtype=np.int64)
        arrays["reduced_data"] = np.asarray(vals)
    else:
        arrays["data"] = np.array(table.data)
    with BytesIO() as f:
        np.savez(f, **arrays)
        return f.getvalue()


def read_payload(blob):
    with BytesIO(blob) as f:
        with np.load(f, allow_pickle=False) as z:
            return {k: z[k] for k in z.files}


class NearFieldInteractionTableManager:
    """Get or build near-field tables through a SQLite cache file."""

    def __init__(self, dataset_filename="nft.sqlite", root_extent=1, dtype=np.float64,
                 read_only="auto", **kwargs):
        self.filename = dataset_filename
        self.root_extent = root_extent
        self.dtype = dtype
        self.table_extra_kwargs = kwargs
        self.last_compute_timings = self.last_load_timings = None
        if read_only == "auto":
            try:
                self._read_only = False
                conn = sqlite3.connect(_uri(dataset_filename, "rwc"), uri=True)
            except sqlite3.OperationalError:
                self._read_only = True
                conn = sqlite3.connect(_uri(dataset_filename, "ro"), uri=True)
        else:
            self._read_only = bool(read_only)
            conn = sqlite3.connect(_uri(dataset_filename, "ro" if read_only else "rwc"),
                                   uri=True)
        conn.row_factory = sqlite3.Row
        conn.execute("PRAGMA foreign_keys = ON")
        self.datafile = conn
        self._init_schema()
        self._check_root_extent()

    # {{{ schema

    def _init_schema(self):
        if not self._read_only:
            self.datafile.executescript("""
            CREATE TABLE IF NOT EXISTS nearfield_cache (
                dim INTEGER NOT NULL, kernel_type TEXT NOT NULL,
                q_order INTEGER NOT NULL, source_box_level INTEGER NOT NULL,
                n_q_points INTEGER NOT NULL, quad_order INTEGER NOT NULL,
                n_pairs INTEGER NOT NULL, source_box_extent REAL NOT NULL,
                source_box_level_stored INTEGER NOT NULL,
                case_encoding_base INTEGER, case_encoding_shift INTEGER,
                build_method TEXT, kernel_type_cached TEXT, payload BLOB,
                PRIMARY KEY (dim, kernel_type, q_order, source_box_level));
            CREATE TABLE IF NOT EXISTS nearfield_cache_kwargs (
                dim INTEGER NOT NULL, kernel_type TEXT NOT NULL,
                q_order INTEGER NOT NULL, source_box_level INTEGER NOT NULL,
                key TEXT NOT NULL, value_type TEXT NOT NULL, value_text TEXT NOT NULL,
                PRIMARY KEY (dim, kernel_type, q_order, source_box_level, key),
                FOREIGN KEY (dim, kernel_type, q_order, source_box_level)
                    REFERENCES nearfield_cache (dim, kernel_type, q_order, source_box_level)
                    ON DELETE CASCADE);
            CREATE TABLE IF NOT EXISTS nearfield_cache_meta (
                key TEXT PRIMARY KEY, value_type TEXT NOT NULL, value_text TEXT NOT NULL);
            """)
        cols = {r["name"] for r in self.datafile.execute("PRAGMA table_info(nearfield_cache)")}
        if "payload" not in cols or cols & {"q_points", "data", "mode_normalizers"}:
            raise RuntimeError(f"the table cache file {self.filename} uses an unsupported "
                               f"schema; rebuild it with schema {TABLE_CACHE_SCHEMA_VERSION}")
        version = self._meta("schema_version")
        if version is None:
            if self._read_only:
                raise RuntimeError(f"{self.filename} is missing schema_version metadata")
            self._set_meta("schema_version", TABLE_CACHE_SCHEMA_VERSION)
            version = TABLE_CACHE_SCHEMA_VERSION
        parts = tuple(int(x) for x in str(version).split("."))
        if parts[0] > int(TABLE_CACHE_SCHEMA_VERSION.split(".")[0]) or parts < (2, 1, 0):
            raise RuntimeError(f"{self.filename} has unsupported schema_version {version}")
        self.cache_schema_version = str(version)
        if not self._read_only:
            self.datafile.commit()

    def _meta(self, key):
        row = self.datafile.execute(
            "SELECT value_type, value_text FROM nearfield_cache_meta WHERE key=?",
            (key,)).fetchone()
        return None if row is None else _text_to_scalar(row["value_type"], row["value_text"])

    def _set_meta(self, key, value):
        ty, text = _scalar_to_text(value)
        self.datafile.execute("INSERT OR REPLACE INTO nearfield_cache_meta "
                              "(key, value_type, value_text) VALUES (?, ?, ?)", (key, ty, text))

    def _check_root_extent(self):
        stored = self._meta("root_extent")
        if stored is None:
            if not self._read_only:
                self._set_meta("root_extent", self.root_extent)
                self.datafile.commit()
            return
        if abs(float(stored) - float(self.root_extent)) >= 1e-15:
            raise RuntimeError(
                f"The table cache file {self.filename} was built with root_extent = "
                f"{stored}, which is different from the requested value {self.root_extent}")

    # }}}

    def _key(self, dim, kernel_type, q_order, source_box_level):
        return (int(dim), str(kernel_type), int(q_order), int(source_box_level))

    def _source_box_extent(self, level):
        return self.root_extent * (2 ** (-int(level)))

    def _kernel(self, dim, kernel_type):
        cls = _KERNELS.get(kernel_type)
        return None if cls is None else cls(dim)

    def get_table(self, dim, kernel_type, q_order, source_box_level=0, force_recompute=False,
                  queue=None, **kwargs):
        key = self._key(dim, kernel_type, q_order, source_box_level)
        row = self.datafile.execute(
            "SELECT 1 FROM nearfield_cache WHERE dim=? AND kernel_type=? AND q_order=? "
            "AND source_box_level=?", key).fetchone()
        if row is not None and not force_recompute:
            try:
                return self._load(key, **kwargs), False
            except KeyError:
                if self._read_only:
                    raise RuntimeError("cached table data is unavailable in read-only mode "
                                       "and cannot be recomputed")
        if self._read_only:
            raise RuntimeError(f"Table cache miss in read-only mode for (dim={key[0]}, "
                               f"kernel_type={key[1]}, q_order={key[2]}, "
                               f"source_box_level={key[3]}).")
        return self._compute_and_store(key, queue=queue, **kwargs), True

    def load_saved_table(self, dim, kernel_type, q_order, source_box_level=0, **kwargs):
        return self._load(self._key(dim, kernel_type, q_order, source_box_level), **kwargs)

    def _load(self, key, **kwargs):
        t0 = time.perf_counter()
        row = self.datafile.execute(
            "SELECT * FROM nearfield_cache WHERE dim=? AND kernel_type=? AND q_order=? "
            "AND source_box_level=?", key).fetchone()
        if row is None:
            raise KeyError("missing table record")
        if row["build_method"] is not None and row["build_method"] != _BUILD_METHOD:
            raise KeyError(f"cached build_method is unsupported; expected {_BUILD_METHOD}")
        if not row["payload"]:
            raise KeyError("table cache payload is missing")
        try:
            p = read_payload(row["payload"])
        except (OSError, EOFError, TypeError, ValueError, zipfile.BadZipFile) as exc:
            raise KeyError("table cache payload is corrupted") from exc
        dim, kernel_type, q, level = key
        dtype = np.asarray(p.get("reduced_data", p.get("data"))).dtype
        table = NearFieldInteractionTable(
            q, dim=dim, sumpy_kernel=self._kernel(dim, kernel_type),
            source_box_extent=self._source_box_extent(level),
            dtype=dtype if np.issubdtype(dtype, np.complexfloating) else self.dtype,
            precomputed_q_points=p["q_points"])
        if abs(table.source_box_extent - row["source_box_extent"]) >= 1e-15 or \
                table.n_q_points != row["n_q_points"] or table.n_pairs != row["n_pairs"]:
            raise KeyError("cache record does not match the requested table")
        if "data" in p:
            table.data = p["data"]
        elif "reduced_entry_ids" in p and "reduced_data" in p:
            table.set_reduced_table_data(p["reduced_entry_ids"], p["reduced_data"])
        else:
            raise KeyError("payload is missing table data arrays")
        table.mode_normalizers[:] = p["mode_normalizers"]
        table.kernel_exterior_normalizers[:] = p["kernel_exterior_normalizers"]
        if not np.array_equal(np.array(table.interaction_case_vecs),
                              p["interaction_case_vecs"]) or \
                not np.array_equal(np.asarray(table.case_indices), p["case_indices"]):
            raise KeyError("cached case gallery differs from this build's")
        table.case_encoding_base = int(row["case_encoding_base"])
        table.case_encoding_shift = int(row["case_encoding_shift"])
        table.source_box_level = level
        table.kernel_type_cached = row["kernel_type_cached"]
        for r in self.datafile.execute(
                "SELECT key, value_type, value_text FROM nearfield_cache_kwargs WHERE dim=? "
                "AND kernel_type=? AND q_order=? AND source_box_level=?", key):
            value = _text_to_scalar(r["value_type"], r["value_text"])
            if r["key"] in kwargs and kwargs[r["key"]] != value:
                raise KeyError(f"cached kernel parameter {r['key']!r} mismatch")
            setattr(table, r["key"], value)
        table.is_built = True
        self.last_load_timings = {"total_s": time.perf_counter() - t0}
        return table

    def _compute_and_store(self, key, queue=None, **kwargs):
        dim, kernel_type, q, level = key
        knl = self._kernel(dim, kernel_type)
        if knl is None:
            raise NotImplementedError(f"no table builder for kernel type {kernel_type!r}")
        dtype = np.complex128 if knl.is_complex_valued else self.dtype
        table = NearFieldInteractionTable(q, dim=dim, sumpy_kernel=knl, dtype=dtype,
                                          source_box_extent=self._source_box_extent(level))
        t0 = time.perf_counter()
        table.build_table(queue=queue, **kwargs)
        t1 = time.perf_counter()
        self.store_table(table, kernel_type, level, **kwargs)
        self.last_compute_timings = {"table_build_s": t1 - t0,
                                     "total_s": time.perf_counter() - t0}
        return table

    def store_table(self, table, kernel_type, source_box_level=0, **kwargs):
        """Store a built table under (table.dim, kernel_type, table.quad_order,
        source_box_level), with its scalar build arguments ``kwargs``."""
        if self._read_only:
            raise RuntimeError("the table cache is open read-only")
        dim, q, level = table.dim, table.quad_order, int(source_box_level)
        key = self._key(dim, kernel_type, q, level)
        if abs(table.source_box_extent - self._source_box_extent(level)) >= 1e-15:
            raise ValueError("the table's source box extent does not match its level")
        vals = sorted({int(c) for v in table.interaction_case_vecs for c in v})
        base, shift = vals[-1] - vals[0] + 1, -vals[0]
        self.datafile.execute(
            "INSERT OR REPLACE INTO nearfield_cache (dim, kernel_type, q_order, "
            "source_box_level, n_q_points, quad_order, n_pairs, source_box_extent, "
            "source_box_level_stored, case_encoding_base, case_encoding_shift, build_method, "
            "kernel_type_cached, payload) VALUES (?, ?, ?, ?, ?, ?, ?, ?, ?, ?, ?, ?, ?, ?)",
            (dim, kernel_type, q, level, table.n_q_points, table.quad_order, table.n_pairs,
             table.source_box_extent, level, base, shift, _BUILD_METHOD, kernel_type,
             table_payload(table)))
        self.datafile.execute(
            "DELETE FROM nearfield_cache_kwargs WHERE dim=? AND kernel_type=? AND q_order=? "
            "AND source_box_level=?", key)
        for name, value in kwargs.items():
            try:
                ty, text = _scalar_to_text(value)
            except TypeError:
                continue
            self.datafile.execute(
                "INSERT INTO nearfield_cache_kwargs (dim, kernel_type, q_order, "
                "source_box_level, key, value_type, value_text) VALUES (?, ?, ?, ?, ?, ?, ?)",
                key + (name, ty, text))
        self.datafile.commit()
        table.source_box_level = level
        table.kernel_type_cached = kernel_type

    def close(self):
        self.datafile.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        if not self._read_only:
            self.datafile.commit()
        self.datafile.close()
