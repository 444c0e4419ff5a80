"""Oracle: CPU restatement of the reference's numeric LBL path (checker and
CPU baseline only; never on the product path)."""
