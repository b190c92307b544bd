"""Generate tests/golden/ref_vectors.npz from the reference's own CPU code.

Run here, where the reference tree is mounted (it is read, never modified):

    python oracle/build.py            # builds oracle/_ref/libiaref.so
    python tests/golden/make_golden.py [<reference CUDA/ directory>]

Contents (all produced by the reference's compiled esm()/ibem()/sphere()/
cartesian_2_spherical(), built with C_AIR=343, RHO_AIR=1.21):
  rule_regular (13, 3), rule_singular (3, 1600, 3)  the reference's quadrature
      tables (CUDA/IPF.txt, CUDA/IPFs.txt), read as golden inputs
  mesh_nodes (3, 42), mesh_elems (3, 80)  icosphere subdiv 1, radius 0.1
  mics (3, 30), chief (3, 2), ks (2,)
  ibem_Z_{0,1}, ibem_H_{0,1}        ibem() at ks[0], ks[1], no CHIEF points
  ibem_chief_Z, ibem_chief_H        ibem() at ks[0] with the 2 CHIEF points
  invr_q, invr_h, invr_m            invr() at ks[1], n_am = m: left singular
      vectors of G Z, (A_hs Z - B_hs) q, Z q
  esm_src (3, 42), esm_fld (3, 42), esm_k, esm_ri, esm_Me, esm_He   esm(), l == m
  kat_ps, kat_ph, kat_u, kat_a     sphere() analytic pressures at mesh nodes / mics
  sph_in (3, 12), sph_out (3, 12)  cartesian_2_spherical()
  msh_k, msh_t, msh_nodes, msh_field, msh_elems   geometry() on tests/golden/sphere42.msh
      (the mesh above as gmsh v2.2 text with 3 point elements and 2 degenerate triangles)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from inverseacoustics_gb300 import geometry as g  # noqa: E402
from oracle import build, ref  # noqa: E402

def main():
    ref_cuda = build.reference_cuda(sys.argv[1] if len(sys.argv) > 1 else None)
    if ref_cuda is None:
        sys.exit("make_golden: the reference's CUDA/ directory was not found "
                 "(pass it as the first argument or set IA_REFERENCE_CUDA)")
    build.build_ref(reference_cuda_dir=ref_cuda)
    c, rho = ref.constants()
    assert (c, rho) == (343.0, 1.21)
    reg, sing = ref.read_reference_rules(ref_cuda)
    rng = np.random.default_rng(1234)
    nodes, elems = g.icosphere(1, 0.10)
    mics = g.hemisphere_array(rng, 30, 0.30)
    chief = np.array([[0.01, 0.02, -0.03], [-0.02, 0.0, 0.015]]).T.copy()
    ks = np.array([2 * np.pi * 400.0 / c, 2 * np.pi * 1500.0 / c])
    out = dict(rule_regular=reg, rule_singular=sing, mesh_nodes=nodes, mesh_elems=elems, mics=mics, chief=chief,
               ks=ks, c=np.array(c), rho=np.array(rho))
    for i, k in enumerate(ks):
        Z, H = ref.ibem(nodes, elems, mics, k, reg, sing)
        out[f"ibem_Z_{i}"], out[f"ibem_H_{i}"] = Z, H
    Z, H = ref.ibem(nodes, elems, mics, ks[0], reg, sing, chief)
    out["ibem_chief_Z"], out["ibem_chief_H"] = Z, H
    # invr() with n_am = m, the one size at which its output products are H U
    # and Z U
    q_e, h_r, m_e = ref.invr(nodes, elems, mics, ks[1], reg, sing, nodes.shape[1])
    out.update(invr_q=q_e, invr_h=h_r, invr_m=m_e)
    src = nodes.copy()
    fld = nodes * 1.8
    esm_k = 2 * np.pi * 800.0 / c
    Me, He = ref.esm(src, fld, esm_k, 0.7)
    out.update(esm_src=src, esm_fld=fld, esm_k=np.array(esm_k), esm_ri=np.array(0.7), esm_Me=Me, esm_He=He)
    ps, ph, _ = ref.sphere(nodes, mics, ks[1], 0.02, 0.10)
    out.update(kat_ps=ps, kat_ph=ph, kat_u=np.array(0.02), kat_a=np.array(0.10))
    P = rng.normal(size=(3, 12))
    out.update(sph_in=P, sph_out=ref.cart2sph(P))
    # gmsh v2.2 file of the same mesh with point elements and degenerate
    # triangles, read by the reference's geometry()
    msh = os.path.join(HERE, "sphere42.msh")
    from oracle import ia_oracle as O
    O.write_msh(msh, nodes, elems, extra_points=3, degenerate=2)
    msh_k, msh_t = 2 * np.pi * 500.0 / c, 0.3
    rn, rl, en = ref.geometry(msh, msh_k, msh_t)
    out.update(msh_k=np.array(msh_k), msh_t=np.array(msh_t), msh_nodes=rn, msh_field=rl, msh_elems=en)
    path = os.path.join(HERE, "ref_vectors.npz")
    np.savez_compressed(path, **out)
    print(path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
