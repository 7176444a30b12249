"""ORACLE — test infrastructure only.

CPU restatement of violet's lighting back end (oracle.cpp) and its build recipe.
Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker; the product package never imports it.
"""
