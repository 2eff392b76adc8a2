"""Example drivers mirroring the reference's src/examples programs (command-line batch runs that
read a mechanism and a scenario file, time the device call and write results in the reference's
text formats)."""
