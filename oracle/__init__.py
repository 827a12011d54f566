"""Oracle package: the CPU restatement of the reference path and the reference's
own host code compiled from source.  Test infrastructure only -- nothing in the
product imports it."""
