"""Oracle package: the CPU restatement (wcfe_oracle.c) and the reference built
from its sources (oracle/_ref).  Test infrastructure only."""
