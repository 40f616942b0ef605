"""The oracle-side workload builder gives the product's benchmark inputs
byte for byte, so the reference leg of the benchmark times the FP64 oracle
on exactly the workload that the GPU leg runs, without loading the product."""
import numpy as np

from oracle import workloads
from pointint_gb300 import configs


def test_matrix256_inputs_identical_to_the_product_builder():
    kg_o, objs_o, meta_o = workloads.matrix256(seed=0)
    kg_p, objs_p, meta_p = configs.matrix256(seed=0)
    assert meta_o == meta_p
    assert len(objs_o) == len(objs_p) == 256
    for a, b in zip(objs_o, objs_p):
        assert a.geom_type == b.geom.type and a.dof_type == b.dof_type
        assert a.elems.tobytes() == b.geom.elems.tobytes()
        assert a.dofs.tobytes() == b.dofs.tobytes()
    for x, y in zip(kg_o, (kg_p.dirs, kg_p.kmag, kg_p.w)):
        assert np.asarray(x).tobytes() == np.asarray(y).tobytes()


def test_matrix256_seeds_differ():
    _, a, _ = workloads.matrix256(seed=1, n_objects=4, with_kgrid=False)
    _, b, _ = workloads.matrix256(seed=2, n_objects=4, with_kgrid=False)
    assert a[0].dofs.tobytes() != b[0].dofs.tobytes()
