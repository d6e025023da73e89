"""TEST ORACLE -- CPU restatements of the reference's algorithms (checker
only).  Imported by tests/, by ``__graft_entry__.smoke()`` and by the CPU
baseline legs of ``bench.py``; never by the product package."""
