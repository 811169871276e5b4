"""Broad Institute file formats: writers for tests and examples, and a loader
that parses through libgsea103 (``gsea_dataset_load``, the reference's
read_gct / read_cls / read_gmt rules)."""
from __future__ import annotations

import ctypes
from typing import List, Sequence, Tuple

import numpy as np

from . import _native as N


def write_gct(path: str, exprs_gm: np.ndarray, genes: Sequence[str], patients: Sequence[str]) -> None:
    """Expression table, gene-major [G][S]; float32 values are written with
    enough digits to parse back exactly."""
    G, S = exprs_gm.shape
    with open(path, "w") as f:
        f.write("#1.2\n")
        f.write(f"{G}\t{S}\n")
        f.write("NAME\tDESCRIPTION\t" + "\t".join(patients) + "\n")
        for g in range(G):
            vals = "\t".join(repr(float(np.float32(v))) for v in exprs_gm[g])
            f.write(f"{genes[g]}\tna\t{vals}\n")


def write_cls(path: str, labels: Sequence[int], names: Tuple[str, str] = ("A", "B")) -> None:
    with open(path, "w") as f:
        f.write(f"{len(labels)} 2 1\n")
        f.write(f"# {names[0]} {names[1]}\n")
        f.write(" ".join(names[int(l)] for l in labels) + "\n")


def write_gmt(path: str, set_names: Sequence[str], sets: Sequence[Sequence[str]]) -> None:
    with open(path, "w") as f:
        for name, members in zip(set_names, sets):
            f.write(name + "\tna\t" + "\t".join(members) + "\n")


class Dataset:
    """A parsed .gct / .cls / .gmt triple (gene-set symbols mapped to indices)."""

    def __init__(self, gct: str, cls: str, gmt: str):
        h = ctypes.c_void_p()
        N.check(N.lib().gsea_dataset_load(gct.encode(), cls.encode(), gmt.encode(), ctypes.byref(h)))
        self._h = h
        dims = [ctypes.c_int64() for _ in range(4)]
        N.check(N.lib().gsea_dataset_dims(h, *[ctypes.byref(x) for x in dims]))
        self.num_genes, self.num_samples, self.num_sets, self.num_members = (x.value for x in dims)

    def arrays(self, precision: int = 32):
        dt = np.float64 if precision == 64 else np.float32
        x = np.empty((self.num_samples, self.num_genes), dt)
        labels = np.empty(self.num_samples, np.uint8)
        off = np.empty(self.num_sets + 1, np.int64)
        genes = np.empty(max(1, self.num_members), np.int32)
        N.check(N.lib().gsea_dataset_arrays(self._h, precision, N.ptr(x), N.ptr(labels), N.ptr(off), N.ptr(genes)))
        return x, labels, off, genes[:self.num_members]

    def gene_symbols(self) -> List[str]:
        return [N.lib().gsea_dataset_gene(self._h, i).decode() for i in range(self.num_genes)]

    def set_names(self) -> List[str]:
        return [N.lib().gsea_dataset_set_name(self._h, k).decode() for k in range(self.num_sets)]

    def close(self):
        if getattr(self, "_h", None):
            N.lib().gsea_dataset_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_dataset(prefix: str, d) -> Tuple[str, str, str]:
    """Write a synthetic GseaInput as <prefix>.gct/.cls/.gmt; returns the paths."""
    genes = d.gene_symbols()
    patients = [f"P{s}" for s in range(d.num_samples)]
    write_gct(prefix + ".gct", d.exprs.T, genes, patients)
    write_cls(prefix + ".cls", d.labels)
    write_gmt(prefix + ".gmt", [f"SET_{k}" for k in range(d.num_sets)], d.set_lists())
    return prefix + ".gct", prefix + ".cls", prefix + ".gmt"


def parse_result_lines(text: str):
    """The CLI's "RESULT: ES: .. NES: .. NP: .. FWER: ..\\t(name)" lines -> (names, [K][4])."""
    names, vals = [], []
    for line in text.splitlines():
        if not line.startswith("RESULT:"):
            continue
        body, name = line.split("\t")
        f = body.split()
        vals.append([float(f[2]), float(f[4]), float(f[6]), float(f[8])])
        names.append(name.strip()[1:-1])
    return names, np.array(vals)
