"""CPU oracle for the generalized-coordinates physics step.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import this package, and only as the
checker (or as the timed CPU restatement); the product path never does.

``oracle.pipeline`` restates brax's generalized pipeline (brax 0.14.2) in numpy,
batched over environments, in float64 or float32.  Two pieces of that pipeline
live in third-party packages that are absent from the reference tree; they are
restated from their published algorithms:

* ``jaxopt.ProjectedGradient`` (unpinned in brax's pyproject.toml:44): FISTA
  proximal gradient with backtracking line search (Beck & Teboulle 2009), as
  used at brax/generalized/constraint.py:229-238;
* the ``mujoco.mjx`` primitive collision functions used through
  brax/contact.py:38,57 (``mujoco>=3.8.1``, ``mujoco-mjx`` unpinned):
  sphere/capsule/box vs plane, sphere-sphere, sphere-capsule and
  capsule-capsule.

Parity status: the restatement is pinned against every literal golden value
of the reference's tests that needs no MuJoCo (actuator, scan, init_q,
sphere-plane / sphere-sphere contact, Newton-Schulz inverse, orthogonals; see
``tests/test_oracle_golden.py``).  The exact jaxopt iterates, the MJX tangent
frames, capsule contact counts and box-plane contacts are *parity unpinned*:
no reference output for them can be produced in this container.
"""
