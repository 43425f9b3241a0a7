"""Oracle for the RAPTOR imaging hot path: TEST INFRASTRUCTURE ONLY.

* oracle/ref.py + ref_driver.c + Makefile: the reference's own C sources,
  compiled unmodified (where they are present) into oracle/_ref/.
* oracle/raptor_port.c + port.py: this project's C restatement of the same
  algorithm, which travels to machines without the reference sources.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this package.  The engine (raptor_gb300) never does.
"""
