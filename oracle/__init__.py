"""Test oracle: CPU restatement of the reference path and a driver for the
compiled reference.  Test infrastructure only -- never imported by the
product package."""
