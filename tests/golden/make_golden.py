"""Regenerate the golden fixtures in this folder from the reference's own tests.

Run once where a checkout of the reference (the scrust repository) exists:

    python tests/golden/make_golden.py <path of the scrust checkout>

It reads the scanpy constants the reference pins in
crates/scrust-core/src/neighbors.rs:498-544 (ten sample cells of
`reference_embedding(300, 20, 42)` with their scanpy neighbour rows and
connectivity rows, and the exact nnz / weight sum / square sum of the whole
matrix) and writes them, unchanged, to `scanpy_reference_embedding_300x20.json`;
and the UMAP constants of crates/scrust-core/src/umap.rs's tests (the 80-cell
scanpy graph and layout, umap-learn's fitted-curve table) to
`umap_reference_80_cells.json`; and scanpy's PCA of the 300 x 200 fixture of
crates/scrust-core/src/pca.rs's tests to `pca_scanpy_300x200.json`.  The
values are parsed from the source text, not re-typed.
"""

from __future__ import annotations

import json
import pathlib
import re
import sys

HERE = pathlib.Path(__file__).resolve().parent


def _block(text: str, name: str) -> str:
    start = text.index(name)
    eq = text.index("=", start)
    end = text.index("];", eq)
    return text[eq + 1 : end + 1]


def _rust_float(token: str) -> float:
    return float(token.replace("_", ""))


def parse(neighbors_rs: str) -> dict:
    cells = [int(v) for v in re.findall(r"\d+", _block(neighbors_rs, "SCANPY_SAMPLE_CELLS"))]
    nb_block = _block(neighbors_rs, "SCANPY_NEIGHBORS")
    rows = re.findall(r"\[([\d,\s]+)\]", nb_block)
    neighbours = [[int(v) for v in re.findall(r"\d+", row)] for row in rows]
    conn_block = _block(neighbors_rs, "SCANPY_CONNECTIVITY_ROWS")
    conn_rows = []
    for row in re.findall(r"&\[(.*?)\]", conn_block, flags=re.S):
        pairs = re.findall(r"\((\d+),\s*([0-9eE_.+-]+)\)", row)
        conn_rows.append([[int(c), _rust_float(v)] for c, v in pairs])
    nnz = int(re.search(r"SCANPY_NNZ:\s*usize\s*=\s*([\d_]+)", neighbors_rs).group(1).replace("_", ""))
    wsum = _rust_float(re.search(r"SCANPY_WEIGHT_SUM:\s*f32\s*=\s*([0-9eE_.+-]+);", neighbors_rs).group(1))
    wsq = _rust_float(
        re.search(r"SCANPY_WEIGHT_SQUARE_SUM:\s*f32\s*=\s*([0-9eE_.+-]+);", neighbors_rs).group(1)
    )
    assert len(cells) == 10 and len(neighbours) == 10 and len(conn_rows) == 10
    assert all(len(r) == 14 for r in neighbours)
    return {
        "source": "crates/scrust-core/src/neighbors.rs:493-544",
        "embedding": {"generator": "splitmix64", "n_cells": 300, "n_dims": 20, "seed": 42},
        "k": 14,
        "sample_cells": cells,
        "scanpy_neighbors": neighbours,
        "scanpy_connectivity_rows": conn_rows,
        "nnz": nnz,
        "weight_sum": wsum,
        "weight_square_sum": wsq,
        "bars": {
            "neighbour_overlap_min_fraction": 0.9,
            "connectivity_relative_tolerance": 1e-3,
            "source": "crates/scrust-core/src/neighbors.rs:546-590",
        },
    }


def parse_umap(umap_rs: str) -> dict:
    """The 80-cell scanpy graph and layout and umap-learn's fitted-curve table
    that crates/scrust-core/src/umap.rs pins (tests module)."""
    n_cells = int(re.search(r"N_CELLS:\s*usize\s*=\s*(\d+)", umap_rs).group(1))
    edges = [[int(h), int(t), _rust_float(w)]
             for h, t, w in re.findall(r"\((\d+),\s*(\d+),\s*([0-9eE_.+-]+)\)", _block(umap_rs, "EDGES: &["))]
    layout = [_rust_float(v) for v in re.findall(r"-?[0-9][0-9eE_.+-]*", _block(umap_rs, "EMBEDDING: &["))]
    table_block = _block(umap_rs, "EXPECTED: &[(f32, f32, f64, f64)]")
    table = [[_rust_float(v) for v in row]
             for row in re.findall(r"\(\s*([0-9eE_.+-]+),\s*([0-9eE_.+-]+),\s*([0-9eE_.+-]+),\s*([0-9eE_.+-]+)\)",
                                   table_block)]
    assert len(layout) == 2 * n_cells and len(table) == 24 and edges
    return {
        "source": "crates/scrust-core/src/umap.rs (tests: reference::EDGES / EMBEDDING, "
                  "fitted_curve_matches_umap_learn::EXPECTED)",
        "n_cells": n_cells,
        "edges_upper": edges,
        "scanpy_layout": layout,
        "fit_ab_table": table,
        "bars": {"fit_ab_relative_tolerance": 1e-4, "near": 15, "wide": 30, "preserved_min_fraction": 0.80,
                 "epochs": 500, "seed": 0},
    }


def parse_pca(pca_rs: str) -> dict:
    """scanpy's arpack PCA of the 300 x 200 LCG fixture that
    crates/scrust-core/src/pca.rs pins (tests module)."""
    ratio = [_rust_float(v) for v in re.findall(r"-?[0-9][0-9eE_.+-]*",
                                                  _block(pca_rs, "SCANPY_VARIANCE_RATIO: [f32; 3]"))]
    variance = [_rust_float(v) for v in re.findall(r"-?[0-9][0-9eE_.+-]*",
                                                     _block(pca_rs, "SCANPY_VARIANCE: [f32; 3]"))]
    start = pca_rs.index("SCANPY_EMBEDDING")
    eq = pca_rs.index("=", start)
    end = pca_rs.index("];", eq)
    rows = re.findall(r"\[([^\[\]]+)\]", pca_rs[eq + 1:end + 1])
    embedding = [[_rust_float(v) for v in re.findall(r"-?[0-9][0-9eE_.+-]*", row)] for row in rows]
    assert len(ratio) == 3 and len(variance) == 3 and len(embedding) == 3 and all(len(r) == 300 for r in embedding)
    return {
        "source": "crates/scrust-core/src/pca.rs (tests: SCANPY_VARIANCE_RATIO, SCANPY_VARIANCE, SCANPY_EMBEDDING; "
                  "scanpy 1.12.2 sc.pp.pca(n_comps=10, svd_solver='arpack'))",
        "fixture": {"generator": "lcg", "seed": 42, "n_cells": 300, "n_genes": 200},
        "scanpy_variance_ratio": ratio,
        "scanpy_variance": variance,
        "scanpy_embedding": embedding,
        "bars": {"correlation_min": 0.99, "variance_relative_tolerance": 1e-3, "n_comps": 10},
    }


def main(argv: list[str]) -> None:
    if len(argv) != 2:
        raise SystemExit("usage: make_golden.py <path of the scrust checkout>")
    root = pathlib.Path(argv[1])
    text = (root / "crates/scrust-core/src/neighbors.rs").read_text()
    out = HERE / "scanpy_reference_embedding_300x20.json"
    out.write_text(json.dumps(parse(text), indent=1) + "\n")
    print(f"wrote {out}")
    umap_text = (root / "crates/scrust-core/src/umap.rs").read_text()
    out = HERE / "umap_reference_80_cells.json"
    out.write_text(json.dumps(parse_umap(umap_text), indent=1) + "\n")
    print(f"wrote {out}")
    pca_text = (root / "crates/scrust-core/src/pca.rs").read_text()
    out = HERE / "pca_scanpy_300x200.json"
    out.write_text(json.dumps(parse_pca(pca_text), indent=1) + "\n")
    print(f"wrote {out}")


if __name__ == "__main__":
    main(sys.argv)
