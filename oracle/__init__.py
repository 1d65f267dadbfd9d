"""Checkers for the HSDL engine (test infrastructure only): the CPU
restatement of the reference path and, where available, the reference's own
CPU code compiled in place."""
